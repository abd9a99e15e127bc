/* Test infrastructure: a driver that runs the CPU oracle (dmc_oracle.c,
 * included whole) on small cases, for a build with AddressSanitizer and
 * UndefinedBehaviorSanitizer.  Any sanitizer report, a non-zero status or a
 * broken invariant makes the program exit non-zero.  It is never part of
 * the product.
 *
 * Cases: every one of the 256 cell configurations (one cell, f32 and u16),
 * samples equal to the isovalue, ragged and degenerate shapes, reversed
 * extents, FP64 mode and smoothing iterations. */
#include "dmc_oracle.c"

#include <stdio.h>

static int fails = 0;
static uint64_t total_vertices = 0, total_quads = 0;

static uint32_t rng_state = 12345u;
static uint32_t rnd(void)
{
    rng_state ^= rng_state << 13;
    rng_state ^= rng_state >> 17;
    rng_state ^= rng_state << 5;
    return rng_state;
}

/* Runs one case and checks the mesh: status 0, quad indices in range, and
 * the vertex array present when vertices exist. */
static void run_case(const char *name, const void *vol, int dtype, const uint32_t dims[3], const float mn[3],
                     const float mx[3], float iso, int precision, uint32_t num_smooth)
{
    oracle_mesh m;
    const int rc = oracle_dmc_ex(vol, dtype, dims, mn, mx, iso, precision, num_smooth, &m);
    if (rc != 0) {
        fprintf(stderr, "%s: status %d\n", name, rc);
        ++fails;
        return;
    }
    if (m.n_vertices && !(precision ? (void *)m.vertices64 : (void *)m.vertices)) {
        fprintf(stderr, "%s: no vertex array\n", name);
        ++fails;
    }
    for (uint64_t i = 0; i < 4 * m.n_quads; ++i)
        if (m.quads[i] >= m.n_vertices) {
            fprintf(stderr, "%s: quad index %u out of %llu vertices\n", name, m.quads[i],
                    (unsigned long long)m.n_vertices);
            ++fails;
            break;
        }
    total_vertices += m.n_vertices;
    total_quads += m.n_quads;
    oracle_free(&m);
}

int main(void)
{
    const float mn[3] = {0.f, 0.f, 0.f}, mx1[3] = {1.f, 1.f, 1.f};
    char name[64];

    /* one cell per configuration: corner i below the isovalue when bit i is
     * set (corner order of the reference: x fastest, then y, then z) */
    for (int cfg = 0; cfg < 256; ++cfg) {
        float vf[8];
        uint16_t vu[8];
        static const int corner_of_point[8] = {0, 1, 3, 2, 4, 5, 7, 6};   /* point (x,y,z) -> cell corner */
        for (int p = 0; p < 8; ++p) {
            const int below = (cfg >> corner_of_point[p]) & 1;
            vf[p] = below ? 0.f : 1.f;
            vu[p] = below ? 100 : 200;
        }
        const uint32_t d2[3] = {2, 2, 2};
        snprintf(name, sizeof name, "config %d f32", cfg);
        run_case(name, vf, 0, d2, mn, mx1, 0.5f, 0, 0);
        snprintf(name, sizeof name, "config %d u16", cfg);
        run_case(name, vu, 1, d2, mn, mx1, 150.f, 0, 0);
    }

    /* random fields with samples equal to the isovalue, ragged shapes */
    static const uint32_t shapes[][3] = {{3, 5, 7}, {17, 13, 11}, {2, 9, 4}, {33, 2, 2}, {1, 4, 4}, {4, 1, 4},
                                         {4, 4, 1}, {2, 2, 2}, {40, 3, 5}};
    for (size_t s = 0; s < sizeof shapes / sizeof shapes[0]; ++s) {
        const uint32_t *d = shapes[s];
        const size_t n = (size_t)d[0] * d[1] * d[2];
        float *vf = (float *)malloc(n * sizeof(float));
        uint16_t *vu = (uint16_t *)malloc(n * sizeof(uint16_t));
        for (size_t i = 0; i < n; ++i) {
            const uint32_t r = rnd() % 3u;   /* below, at, above the isovalue */
            vf[i] = r == 0 ? -1.f : (r == 1 ? 0.25f : 2.f);
            vu[i] = (uint16_t)(r == 0 ? 7 : (r == 1 ? 40 : 9000));
        }
        const float lo[3] = {-2.f, 1.f, 3.f}, hi[3] = {2.f, -1.f, 9.f};   /* one reversed axis */
        for (int prec = 0; prec < 2; ++prec) {
            snprintf(name, sizeof name, "shape %zu f32 prec %d", s, prec);
            run_case(name, vf, 0, d, lo, hi, 0.25f, prec, 0);
            snprintf(name, sizeof name, "shape %zu u16 prec %d", s, prec);
            run_case(name, vu, 1, d, lo, hi, 40.f, prec, 0);
        }
        snprintf(name, sizeof name, "shape %zu f32 smoothed", s);
        run_case(name, vf, 0, d, lo, hi, 0.25f, 0, 3);
        free(vf);
        free(vu);
    }

    /* a smooth field with many active cells, smoothed */
    {
        const uint32_t d[3] = {21, 21, 21};
        float *vf = (float *)malloc(21 * 21 * 21 * sizeof(float));
        for (int z = 0; z < 21; ++z)
            for (int y = 0; y < 21; ++y)
                for (int x = 0; x < 21; ++x)
                    vf[(z * 21 + y) * 21 + x] = (float)((x - 10) * (x - 10) + (y - 10) * (y - 10) + (z - 10) * (z - 10));
        const float lo[3] = {-5.f, -5.f, -5.f}, hi[3] = {5.f, 5.f, 5.f};
        run_case("sphere smoothed", vf, 0, d, lo, hi, 16.81f, 0, 15);
        free(vf);
    }

    /* argument errors are reported, not crashed on */
    {
        oracle_mesh m;
        const uint32_t d[3] = {2, 2, 2};
        if (oracle_dmc(NULL, 0, d, mn, mx1, 0.f, 0, &m) != 1) {
            fprintf(stderr, "null volume not rejected\n");
            ++fails;
        }
    }

    if (fails) {
        fprintf(stderr, "%d failures\n", fails);
        return 1;
    }
    printf("sanitize check: ok (%llu vertices, %llu quads)\n", (unsigned long long)total_vertices,
           (unsigned long long)total_quads);
    return 0;
}
