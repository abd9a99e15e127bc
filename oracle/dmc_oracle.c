/*
 * CPU oracle for Dual Marching Cubes — TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, step by step, the algorithm of the reference
 * implementation (vcg-thin-meshgen/Framework, DMC_CUDA/DMC_CUDA/src/dmc.cu,
 * function dmc::run_dmc at dmc.cu:2069-2208) as plain sequential C, so that
 * the CUDA extractor in framework_gb300/csrc can be checked against it.  It is
 * only ever loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline; the product never calls it.
 *
 * Parity pin: the reference has no tests and no golden outputs for this path.
 * This restatement is pinned by (a) the lookup tables, which are checked byte
 * for byte against the reference's tables, (b) hand-built single-cell and
 * two-cell cases whose expected output is derived by hand in tests/, and
 * (c) the golden fixtures in tests/golden, produced by this oracle and checked
 * for mesh invariants (closed 2-manifold, Euler characteristic).  No run of the
 * reference itself backs it: the reference is CUDA-only and cannot execute in
 * the build container.
 *
 * Two arithmetic modes:
 *   precision 0 — FP32 replica: every float operation in the order the
 *                 reference performs it, without fused multiply-add
 *                 (compile with -ffp-contract=off).  This is the bit-exact
 *                 target for the GPU.
 *   precision 1 — FP64: the same topology, positions evaluated in double.
 *
 * Deliberate, documented divergences from the reference (two).  First, an
 * owned edge whose endpoints are "bipolar" by the reference's test
 * (dmc.cu:1101-1106) but fall on the same side of the config bits (one sample
 * equals the isovalue, the other is above it) gets its edge vertex emitted as
 * in the reference, but no quad: the reference would look up NO_VERTEX (0xff)
 * in the ring cells (or read outside the compact array for an inactive ring
 * cell), producing an invalid index.  Such quads are counted in
 * n_dropped_quads.  Second, a dual vertex whose patch has no owner cell
 * inside the volume gets the mean of its patch's crossings computed locally,
 * where the reference leaves it uninitialised (dmc.cu:1584-1592).  Samples
 * that are NaN are not supported.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../framework_gb300/csrc/dmc_tables.inc"

#define INVALID32 0xFFFFFFFFu
#define SCAN_BLOCK 65536u   /* cells per block of the parallel exclusive scans */

typedef struct {
    float *vertices;      /* 3 * n_vertices (precision 0) */
    double *vertices64;   /* 3 * n_vertices (precision 1) */
    uint32_t *quads;      /* 4 * n_quads */
    uint64_t n_vertices;
    uint64_t n_quads;
    uint64_t n_active;
    uint64_t n_lut2;
    uint64_t n_dropped_quads;
    uint64_t n_iso_samples;
    uint8_t *ownerless;   /* per vertex (precision 0): 1 for a dual vertex whose patch has no
                             edge with an owner cell inside the volume (the reference leaves
                             those uninitialised, dmc.cu:1584-1592), else 0 */
} oracle_mesh;

/* per active cell record, after _VoxelInfo (dmc.cu:814-1006) */
typedef struct {
    uint64_t index1d;
    uint32_t vertex_begin;
    uint8_t config;
    uint8_t info;   /* bit0-2: edge 6/9/10 bipolar, bit3-5: ccw, bit7: lut2 */
    uint8_t nv;
    uint8_t pad;
} cell_rec;

typedef struct {
    const void *vol;
    int dtype;            /* 0 float32, 1 uint16 */
    uint64_t nx, ny;      /* point dims */
    uint64_t cx, cy, cz;  /* cell dims */
} grid;

static inline float sample(const grid *g, uint64_t x, uint64_t y, uint64_t z)
{
    uint64_t i = (z * g->ny + y) * g->nx + x;
    if (g->dtype == 1) return (float)((const uint16_t *)g->vol)[i];
    return ((const float *)g->vol)[i];
}

/* corner c of cell (x,y,z): dmc.cu:1044-1054 */
static inline void corners(const grid *g, uint64_t x, uint64_t y, uint64_t z, float v[8])
{
    v[0] = sample(g, x, y, z);         v[1] = sample(g, x + 1, y, z);
    v[2] = sample(g, x + 1, y + 1, z); v[3] = sample(g, x, y + 1, z);
    v[4] = sample(g, x, y, z + 1);     v[5] = sample(g, x + 1, y, z + 1);
    v[6] = sample(g, x + 1, y + 1, z + 1); v[7] = sample(g, x, y + 1, z + 1);
}

/* dmc.cu:1018-1027 */
static inline uint8_t config_of(const float v[8], float iso)
{
    uint8_t m = 0;
    for (int i = 0; i < 8; ++i) m |= (uint8_t)((v[i] < iso) << i);
    return m;
}

/* dmc.cu:1101-1106 */
static inline int ref_bipolar(float a, float b, float iso)
{
    if (a == b) return 0;
    if (a > b) { float t = a; a = b; b = t; }
    return !((a < iso && b < iso) || (a > iso && b > iso));
}

/* utils.hpp:118-122: (float)i / size * range + min, no contraction */
static inline float ijk_to_xyz(uint64_t i, uint64_t size, float range, float mn)
{
    float q = (float)i / (float)size;
    float p = q * range;
    return p + mn;
}
static inline double ijk_to_xyz64(uint64_t i, uint64_t size, double range, double mn)
{
    return (double)i / (double)size * range + mn;
}

/* dmc.cu:1090-1098 */
static inline void lerp3(const float p0[3], const float p1[3], float v0, float v1, float iso, float out[3])
{
    float t = (iso - v0) / (v1 - v0);
    float omt = 1.0f - t;
    for (int c = 0; c < 3; ++c) {
        float a = p0[c] * omt;
        float b = p1[c] * t;
        out[c] = a + b;
    }
}
static inline void lerp3_64(const double p0[3], const double p1[3], double v0, double v1, double iso, double out[3])
{
    double t = (iso - v0) / (v1 - v0);
    for (int c = 0; c < 3; ++c) out[c] = p0[c] * (1.0 - t) + p1[c] * t;
}

/* edge_belonged_voxel_lut (dmc.cu:634-649) decoded: offset to the owner cell
 * (each component 0 or -1) and the owner's edge (6, 9 or 10) */
static const int8_t OWNER_OFF[12][3] = {
    {0, -1, -1}, {0, 0, -1}, {0, 0, -1}, {-1, 0, -1}, {-1, -1, 0}, {0, -1, 0},
    {0, 0, 0},   {-1, 0, 0}, {0, -1, 0}, {0, 0, 0},   {0, 0, 0},   {-1, 0, 0}};
static const uint8_t OWNER_EDGE[12] = {10, 9, 10, 9, 6, 6, 6, 6, 10, 9, 10, 9};

/* circular_edge_lut (dmc.cu:653-658): edges around owned edge 6/9/10 in ccw order */
static const uint8_t RING[3][4] = {{6, 7, 4, 5}, {9, 1, 3, 11}, {10, 8, 0, 2}};

/* corner offsets and edge endpoints (dmc.cu:1109-1129) */
static const uint8_t CORNER_OFF[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};
static const uint8_t EDGE_PTS[12][2] = {{0,1},{1,2},{2,3},{0,3},{0,4},{1,5},{2,6},{3,7},{4,5},{5,6},{6,7},{4,7}};

/* endpoints of edge e ordered along the edge's axis (lower coordinate first) */
static void edge_lo_hi(int e, int *lo, int *hi)
{
    int a = EDGE_PTS[e][0], b = EDGE_PTS[e][1];
    int axis = OWNER_EDGE[e] == 10 ? 0 : (OWNER_EDGE[e] == 9 ? 1 : 2);
    if (CORNER_OFF[a][axis] < CORNER_OFF[b][axis]) { *lo = a; *hi = b; } else { *lo = b; *hi = a; }
}

/* Crossing of edge e of cell (x,y,z) computed in the orientation its owner uses
 * (owner edge 6: low z -> high z; 9: low y -> high y; 10: high x -> low x).
 * Used only for a dual vertex whose patch has no edge with an in-volume owner:
 * the reference never writes such a vertex (it is unreferenced and left
 * uninitialised, dmc.cu:1584-1592); here it gets the mean of these crossings. */
static void crossing_local(const grid *g, uint64_t x, uint64_t y, uint64_t z, int e, float iso,
                           const float rng[3], const float mn[3], const uint64_t csz[3], float out[3])
{
    int oe = OWNER_EDGE[e];
    int lo, hi;
    edge_lo_hi(e, &lo, &hi);
    int first = (oe == 10) ? hi : lo, second = (oe == 10) ? lo : hi;
    uint64_t q0[3] = {x + CORNER_OFF[first][0], y + CORNER_OFF[first][1], z + CORNER_OFF[first][2]};
    uint64_t q1[3] = {x + CORNER_OFF[second][0], y + CORNER_OFF[second][1], z + CORNER_OFF[second][2]};
    float p0[3], p1[3];
    for (int c = 0; c < 3; ++c) { p0[c] = ijk_to_xyz(q0[c], csz[c], rng[c], mn[c]); p1[c] = ijk_to_xyz(q1[c], csz[c], rng[c], mn[c]); }
    lerp3(p0, p1, sample(g, q0[0], q0[1], q0[2]), sample(g, q1[0], q1[1], q1[2]), iso, out);
}
static void crossing_local64(const grid *g, uint64_t x, uint64_t y, uint64_t z, int e, double iso,
                             const double rng[3], const float mn[3], const uint64_t csz[3], double out[3])
{
    int oe = OWNER_EDGE[e];
    int lo, hi;
    edge_lo_hi(e, &lo, &hi);
    int first = (oe == 10) ? hi : lo, second = (oe == 10) ? lo : hi;
    uint64_t q0[3] = {x + CORNER_OFF[first][0], y + CORNER_OFF[first][1], z + CORNER_OFF[first][2]};
    uint64_t q1[3] = {x + CORNER_OFF[second][0], y + CORNER_OFF[second][1], z + CORNER_OFF[second][2]};
    double p0[3], p1[3];
    for (int c = 0; c < 3; ++c) { p0[c] = ijk_to_xyz64(q0[c], csz[c], rng[c], mn[c]); p1[c] = ijk_to_xyz64(q1[c], csz[c], rng[c], mn[c]); }
    lerp3_64(p0, p1, sample(g, q0[0], q0[1], q0[2]), sample(g, q1[0], q1[1], q1[2]), iso, out);
}

static inline int owned_slot(int e) { return e == 6 ? 0 : (e == 9 ? 1 : 2); }

/* _VoxelInfo::edge_vertex_index (dmc.cu:911-921) */
static inline uint32_t edge_vertex_index(const cell_rec *r, int e)
{
    int s = owned_slot(e);
    uint32_t off = 0;
    for (int i = 0; i < s; ++i) off += (r->info >> i) & 1u;
    uint32_t n_edge = (r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u);
    return r->vertex_begin + (uint32_t)(r->nv - n_edge) + off;
}

static inline uint8_t lut_m(const cell_rec *r, int e)
{
    return (r->info & 0x80) ? DMC_EDGE_LUT2[r->config * 12 + e] : DMC_EDGE_LUT1[r->config * 12 + e];
}

void oracle_free(oracle_mesh *m)
{
    if (!m) return;
    free(m->vertices); free(m->vertices64); free(m->quads); free(m->ownerless);
    m->vertices = NULL; m->vertices64 = NULL; m->quads = NULL; m->ownerless = NULL;
}

const char *oracle_tables_sha256(void) { return DMC_TABLES_SHA256; }

void oracle_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ---- vertex smoothing (dmc.cu:1710-1981, driven at 2157-2169) ----------
 *
 * One iteration moves the crossing of every owned edge that has a quad onto
 * the split triangle of its ring of four dual vertices, projected along the
 * edge's axis, then recomputes every dual vertex as the mean of its patch's
 * (moved) crossings.  Arithmetic, shared bit for bit with the CUDA kernels:
 * single precision without fused multiply-add, correctly rounded square root
 * and division, the reference's operand order.  Two restatements of the
 * reference's arithmetic (documented divergences): vector lengths are
 * normalised with 1/sqrt (the reference uses the approximate rsqrtf), and the
 * diagonal of a convex quadrilateral is chosen at the corner with the
 * smallest cosine instead of the largest acosf angle (the same corner except
 * where acosf rounds two cosines to one angle). */

/* sign of the z component of (right - mid) x (left - mid) (dmc.cu:1742-1748) */
static inline int cross_z_positive(const float l[2], const float m[2], const float r[2])
{
    float dx1 = r[0] - m[0], dy1 = r[1] - m[1];
    float dx2 = l[0] - m[0], dy2 = l[1] - m[1];
    float a = dx1 * dy2, b = dx2 * dy1;
    return (a - b) >= 0.0f;
}

/* cosine of the angle at m between m->l and m->r (calc_radian without acosf, dmc.cu:1833-1843) */
static inline float corner_cos(const float l[2], const float m[2], const float r[2])
{
    float ux = l[0] - m[0], uy = l[1] - m[1], vx = r[0] - m[0], vy = r[1] - m[1];
    float iu = 1.0f / sqrtf(ux * ux + uy * uy), iv = 1.0f / sqrtf(vx * vx + vy * vy);
    ux = ux * iu; uy = uy * iu; vx = vx * iv; vy = vy * iv;
    return ux * vx + uy * vy;
}

/* is_inside_triangle (dmc.cu:1894-1912): barycentric (alpha, beta, gamma) of pt */
static inline int inside_triangle(const float p0[2], const float p1[2], const float p2[2], const float pt[2],
                                  float *alpha, float *beta, float *gamma)
{
    float v0x = p1[0] - p0[0], v0y = p1[1] - p0[1];
    float v1x = p2[0] - p0[0], v1y = p2[1] - p0[1];
    float v2x = pt[0] - p0[0], v2y = pt[1] - p0[1];
    float d00 = v0x * v0x + v0y * v0y;
    float d10 = v1x * v0x + v1y * v0y;
    float d11 = v1x * v1x + v1y * v1y;
    float d20 = v2x * v0x + v2y * v0y;
    float d21 = v2x * v1x + v2y * v1y;
    float denom = d00 * d11 - d10 * d10;
    float inv = 1.0f / denom;
    *beta = (d11 * d20 - d10 * d21) * inv;
    *gamma = (d00 * d21 - d10 * d20) * inv;
    *alpha = 1.0f - *beta - *gamma;
    float bg = *beta + *gamma;
    return (-1e-4 < (double)*beta) && (-1e-4 < (double)*gamma) && ((double)bg < 1.0 + 1e-4);
}

/* smooth_edge_vertices for one owned edge (axis s: 0 = edge 6, 1 = 9, 2 = 10)
 * whose quad ring holds dual vertices ring[0..3]; origin is the edge's
 * position in the projection plane.  Returns 1 and the new crossing in out
 * when it moves. */
static int smooth_edge(const float *vt, const uint32_t ring[4], int s, const float origin[2], float out[3])
{
    const int ax = s == 2 ? 1 : 0, ay = s == 0 ? 1 : 2;     /* 6: xy, 9: xz, 10: yz */
    float P[4][2];
    for (int i = 0; i < 4; ++i) { P[i][0] = vt[3 * (uint64_t)ring[i] + ax]; P[i][1] = vt[3 * (uint64_t)ring[i] + ay]; }
    int npos = 0, nneg = 0, ipos = 0, ineg = 0;
    for (int i = 0; i < 4; ++i) {
        if (cross_z_positive(P[(i + 3) & 3], P[i], P[(i + 1) & 3])) { npos++; ipos = i; }
        else { nneg++; ineg = i; }
    }
    if (npos == nneg) return 0;                              /* complex quadrilateral */
    int split0;
    if (npos == 0 || nneg == 0) {                             /* convex: corner with the widest angle */
        float best = corner_cos(P[3], P[0], P[1]);
        split0 = 0;
        for (int i = 1; i < 4; ++i) {
            float c = corner_cos(P[(i + 3) & 3], P[i], P[(i + 1) & 3]);
            if (c < best) { best = c; split0 = i; }
        }
    } else {
        split0 = npos < nneg ? ipos : ineg;                  /* the concave corner */
    }
    int split1 = (split0 + 2) & 3;
    float al, be, ga;
    int a, b, c;
    if (inside_triangle(P[split0], P[(split0 + 1) & 3], P[split1], origin, &al, &be, &ga)) {
        a = split0; b = (split0 + 1) & 3; c = split1;
    } else if (inside_triangle(P[split1], P[(split1 + 1) & 3], P[split0], origin, &al, &be, &ga)) {
        a = split1; b = (split1 + 1) & 3; c = split0;
    } else {
        return 0;
    }
    for (int k = 0; k < 3; ++k) {
        float t = al * vt[3 * (uint64_t)ring[a] + k];
        t = t + be * vt[3 * (uint64_t)ring[b] + k];
        t = t + ga * vt[3 * (uint64_t)ring[c] + k];
        out[k] = t;
    }
    return 1;
}

int oracle_dmc_ex(const void *vol, int dtype, const uint32_t dims[3], const float xyz_min[3],
                  const float xyz_max[3], float iso, int precision, uint32_t num_smooth, oracle_mesh *out);

/* Returns 0 on success, 1 bad argument, 2 out of memory, 3 more than 2^32-1
 * vertices (the reference indexes vertices with 32-bit integers). */
int oracle_dmc(const void *vol, int dtype, const uint32_t dims[3],
               const float xyz_min[3], const float xyz_max[3], float iso,
               int precision, oracle_mesh *out)
{
    return oracle_dmc_ex(vol, dtype, dims, xyz_min, xyz_max, iso, precision, 0, out);
}

/* oracle_dmc with num_smooth smoothing iterations (FP32 replica only). */
int oracle_dmc_ex(const void *vol, int dtype, const uint32_t dims[3], const float xyz_min[3],
                  const float xyz_max[3], float iso, int precision, uint32_t num_smooth, oracle_mesh *out)
{
    memset(out, 0, sizeof(*out));
    if (!vol || (dtype != 0 && dtype != 1) || (precision != 0 && precision != 1)) return 1;
    if (precision == 1 && num_smooth) return 1;
    grid g;
    g.vol = vol; g.dtype = dtype;
    g.nx = dims[0]; g.ny = dims[1];
    if (dims[0] < 2 || dims[1] < 2 || dims[2] < 2) return 0;   /* no cells: empty mesh */
    g.cx = dims[0] - 1; g.cy = dims[1] - 1; g.cz = dims[2] - 1;
    const uint64_t C = g.cx * g.cy * g.cz;
    const uint64_t N = (uint64_t)dims[0] * dims[1] * dims[2];

    {   /* samples exactly at the isovalue (for test pre-screening) */
        uint64_t cnt = 0;
        #pragma omp parallel for reduction(+:cnt) schedule(static)
        for (int64_t i = 0; i < (int64_t)N; ++i) {
            float v = dtype == 1 ? (float)((const uint16_t *)vol)[i] : ((const float *)vol)[i];
            cnt += (v == iso);
        }
        out->n_iso_samples = cnt;
    }

    /* step 2: flag + compact active cells in index1D order (dmc.cu:1035-1158).
     * The flag pass runs per z-slice in parallel; the compaction is sequential. */
    uint32_t *map = (uint32_t *)malloc(C * sizeof(uint32_t));   /* full_voxel_index_map */
    uint8_t *cfg = (uint8_t *)malloc(C);
    if (!map || !cfg) { free(map); free(cfg); return 2; }
    #pragma omp parallel for schedule(dynamic, 1)
    for (int64_t z = 0; z < (int64_t)g.cz; ++z)
        for (uint64_t y = 0; y < g.cy; ++y)
            for (uint64_t x = 0; x < g.cx; ++x) {
                float v[8];
                corners(&g, x, y, (uint64_t)z, v);
                cfg[((uint64_t)z * g.cy + y) * g.cx + x] = config_of(v, iso);
            }
    /* Active cells numbered in index1D order, exactly as one serial pass
     * would: per-block counts in parallel, an exclusive prefix over the
     * blocks, then each block numbers its own cells. */
    const uint64_t nblk = (C + SCAN_BLOCK - 1) / SCAN_BLOCK;
    uint64_t *boff = (uint64_t *)calloc(nblk + 1, sizeof(uint64_t));
    if (!boff) { free(map); free(cfg); return 2; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk; ++b) {
        const uint64_t i0 = (uint64_t)b * SCAN_BLOCK, i1 = i0 + SCAN_BLOCK < C ? i0 + SCAN_BLOCK : C;
        uint64_t n = 0;
        for (uint64_t i = i0; i < i1; ++i) n += (cfg[i] != 0 && cfg[i] != 0xff);
        boff[b + 1] = n;
    }
    for (uint64_t b = 0; b < nblk; ++b) boff[b + 1] += boff[b];
    const uint64_t A = boff[nblk];
    if (A >= INVALID32) { free(boff); free(map); free(cfg); return 3; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk; ++b) {
        const uint64_t i0 = (uint64_t)b * SCAN_BLOCK, i1 = i0 + SCAN_BLOCK < C ? i0 + SCAN_BLOCK : C;
        uint64_t k = boff[b];
        for (uint64_t i = i0; i < i1; ++i) map[i] = (cfg[i] != 0 && cfg[i] != 0xff) ? (uint32_t)k++ : INVALID32;
    }
    out->n_active = A;
    cell_rec *rec = (cell_rec *)calloc(A ? A : 1, sizeof(cell_rec));
    if (!rec) { free(boff); free(map); free(cfg); return 2; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk; ++b) {
        const uint64_t i0 = (uint64_t)b * SCAN_BLOCK, i1 = i0 + SCAN_BLOCK < C ? i0 + SCAN_BLOCK : C;
        for (uint64_t i = i0; i < i1; ++i)
            if (map[i] != INVALID32) rec[map[i]].index1d = i;
    }
    free(boff);

    /* step 3: config + bipolar/ccw bits of owned edges 6 (2-6), 9 (5-6), 10 (7-6)
     * (dmc.cu:1173-1221) */
    #pragma omp parallel for schedule(static)
    for (int64_t a = 0; a < (int64_t)A; ++a) {
        cell_rec *r = &rec[a];
        uint64_t i1 = r->index1d;
        uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
        float v[8];
        corners(&g, x, y, z, v);
        r->config = config_of(v, iso);
        static const int P0[3] = {2, 5, 7};
        uint8_t info = 0;
        for (int s = 0; s < 3; ++s) {
            if (ref_bipolar(v[P0[s]], v[6], iso)) {
                info |= (uint8_t)(1u << s);
                if (v[P0[s]] <= iso) info |= (uint8_t)(1u << (s + 3));
            }
        }
        r->info = info;
    }

    /* step 4: 2B/3B correction (dmc.cu:1232-1371).  The neighbour across the
     * ambiguous face shares that face's alternating corners, so it is active. */
    uint64_t n_lut2 = 0;
    #pragma omp parallel for reduction(+:n_lut2) schedule(static)
    for (int64_t a = 0; a < (int64_t)A; ++a) {
        cell_rec *r = &rec[a];
        uint8_t face = DMC_AMBIGUOUS_FACE[r->config];
        if (face == 0xff) continue;
        uint64_t i1 = r->index1d;
        int64_t x = (int64_t)(i1 % g.cx), y = (int64_t)((i1 / g.cx) % g.cy), z = (int64_t)(i1 / (g.cx * g.cy));
        int dir = DMC_FACE_DIR[face];
        int64_t nx_ = x, ny_ = y, nz_ = z;
        switch (dir) {
            case 0: nx_ = x + 1; break; case 1: nx_ = x - 1; break;
            case 2: ny_ = y + 1; break; case 3: ny_ = y - 1; break;
            case 4: nz_ = z + 1; break; default: nz_ = z - 1; break;
        }
        if (nx_ < 0 || ny_ < 0 || nz_ < 0 || nx_ >= (int64_t)g.cx || ny_ >= (int64_t)g.cy || nz_ >= (int64_t)g.cz)
            continue;
        uint64_t ni = ((uint64_t)nz_ * g.cy + (uint64_t)ny_) * g.cx + (uint64_t)nx_;
        uint8_t ncfg = cfg[ni];
        if (DMC_AMBIGUOUS_FACE[ncfg] != 0xff) { r->info |= 0x80; n_lut2++; }
    }
    out->n_lut2 = n_lut2;

    /* step 5: vertex counts and offsets (dmc.cu:1382-1424, 2133-2141): the
     * counts in parallel, then the same blocked exclusive scan */
    #pragma omp parallel for schedule(static)
    for (int64_t a = 0; a < (int64_t)A; ++a) {
        cell_rec *r = &rec[a];
        uint8_t n = (r->info & 0x80) ? DMC_NVERT_LUT2[r->config] : DMC_NVERT_LUT1[r->config];
        r->nv = (uint8_t)(n + (r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u));
    }
    const uint64_t nblk_a = (A + SCAN_BLOCK - 1) / SCAN_BLOCK;
    uint64_t *aoff = (uint64_t *)calloc(nblk_a + 1, sizeof(uint64_t));
    if (!aoff) { free(map); free(cfg); free(rec); return 2; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk_a; ++b) {
        const uint64_t a0 = (uint64_t)b * SCAN_BLOCK, a1 = a0 + SCAN_BLOCK < A ? a0 + SCAN_BLOCK : A;
        uint64_t n = 0;
        for (uint64_t a = a0; a < a1; ++a) n += rec[a].nv;
        aoff[b + 1] = n;
    }
    for (uint64_t b = 0; b < nblk_a; ++b) aoff[b + 1] += aoff[b];
    const uint64_t V = aoff[nblk_a];
    if (V > INVALID32) { free(aoff); free(map); free(cfg); free(rec); return 3; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk_a; ++b) {
        const uint64_t a0 = (uint64_t)b * SCAN_BLOCK, a1 = a0 + SCAN_BLOCK < A ? a0 + SCAN_BLOCK : A;
        uint64_t v = aoff[b];
        for (uint64_t a = a0; a < a1; ++a) { rec[a].vertex_begin = (uint32_t)v; v += rec[a].nv; }
    }
    out->n_vertices = V;

    /* step 6: geometry */
    const float rng[3] = {xyz_max[0] - xyz_min[0], xyz_max[1] - xyz_min[1], xyz_max[2] - xyz_min[2]};
    const uint64_t csz[3] = {g.cx, g.cy, g.cz};
    if (precision == 0) {
        float *vt = (float *)malloc((V ? V : 1) * 3 * sizeof(float));
        uint8_t *own = (uint8_t *)calloc(V ? V : 1, 1);
        if (!vt || !own) { free(vt); free(own); free(aoff); free(map); free(cfg); free(rec); return 2; }
        out->vertices = vt;
        out->ownerless = own;
        /* edge crossings on owned edges (dmc.cu:1468-1514) */
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
            uint32_t vi = r->vertex_begin + r->nv - ((r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u));
            float x1 = ijk_to_xyz(x + 1, csz[0], rng[0], xyz_min[0]);
            float y1 = ijk_to_xyz(y + 1, csz[1], rng[1], xyz_min[1]);
            float z1 = ijk_to_xyz(z + 1, csz[2], rng[2], xyz_min[2]);
            float v6 = sample(&g, x + 1, y + 1, z + 1);
            if (r->info & 1u) {
                float p0[3] = {x1, y1, ijk_to_xyz(z, csz[2], rng[2], xyz_min[2])}, p1[3] = {x1, y1, z1};
                lerp3(p0, p1, sample(&g, x + 1, y + 1, z), v6, iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
            if (r->info & 2u) {
                float p0[3] = {x1, ijk_to_xyz(y, csz[1], rng[1], xyz_min[1]), z1}, p1[3] = {x1, y1, z1};
                lerp3(p0, p1, sample(&g, x + 1, y, z + 1), v6, iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
            if (r->info & 4u) {
                float p0[3] = {x1, y1, z1}, p1[3] = {ijk_to_xyz(x, csz[0], rng[0], xyz_min[0]), y1, z1};
                lerp3(p0, p1, v6, sample(&g, x, y + 1, z + 1), iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
        }
        /* dual vertices: mean of the crossings of the patch (dmc.cu:1517-1593),
         * accumulated in edge order: first assign, then +=, then /= count */
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            int64_t x = (int64_t)(i1 % g.cx), y = (int64_t)((i1 / g.cx) % g.cy), z = (int64_t)(i1 / (g.cx * g.cy));
            uint8_t cnt[4] = {0, 0, 0, 0};
            for (int e = 0; e < 12; ++e) {
                uint8_t m = lut_m(r, e);
                if (m == 0xff) continue;
                int64_t ox = x + OWNER_OFF[e][0], oy = y + OWNER_OFF[e][1], oz = z + OWNER_OFF[e][2];
                if (ox < 0 || oy < 0 || oz < 0) continue;
                uint64_t oi = ((uint64_t)oz * g.cy + (uint64_t)oy) * g.cx + (uint64_t)ox;
                const cell_rec *owner = &rec[map[oi]];
                const float *src = &vt[3 * (uint64_t)edge_vertex_index(owner, OWNER_EDGE[e])];
                float *dst = &vt[3 * ((uint64_t)r->vertex_begin + m)];
                if (cnt[m] == 0) { dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; }
                else { dst[0] = dst[0] + src[0]; dst[1] = dst[1] + src[1]; dst[2] = dst[2] + src[2]; }
                cnt[m]++;
            }
            uint8_t niso = (uint8_t)(r->nv - ((r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u)));
            for (uint8_t m = 0; m < niso; ++m) {
                float *dst = &vt[3 * ((uint64_t)r->vertex_begin + m)];
                if (!cnt[m]) {
                    own[(uint64_t)r->vertex_begin + m] = 1;
                    for (int e = 0; e < 12; ++e) {
                        if (lut_m(r, e) != m) continue;
                        float c3[3];
                        crossing_local(&g, (uint64_t)x, (uint64_t)y, (uint64_t)z, e, iso, rng, xyz_min, csz, c3);
                        if (cnt[m] == 0) { dst[0] = c3[0]; dst[1] = c3[1]; dst[2] = c3[2]; }
                        else { dst[0] = dst[0] + c3[0]; dst[1] = dst[1] + c3[1]; dst[2] = dst[2] + c3[2]; }
                        cnt[m]++;
                    }
                }
                float d = (float)cnt[m];
                dst[0] = dst[0] / d; dst[1] = dst[1] / d; dst[2] = dst[2] / d;
            }
        }
    } else {
        double *vt = (double *)malloc((V ? V : 1) * 3 * sizeof(double));
        if (!vt) { free(aoff); free(map); free(cfg); free(rec); return 2; }
        out->vertices64 = vt;
        const double rng64[3] = {(double)xyz_max[0] - xyz_min[0], (double)xyz_max[1] - xyz_min[1], (double)xyz_max[2] - xyz_min[2]};
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
            uint32_t vi = r->vertex_begin + r->nv - ((r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u));
            double x1 = ijk_to_xyz64(x + 1, csz[0], rng64[0], xyz_min[0]);
            double y1 = ijk_to_xyz64(y + 1, csz[1], rng64[1], xyz_min[1]);
            double z1 = ijk_to_xyz64(z + 1, csz[2], rng64[2], xyz_min[2]);
            double v6 = sample(&g, x + 1, y + 1, z + 1);
            if (r->info & 1u) {
                double p0[3] = {x1, y1, ijk_to_xyz64(z, csz[2], rng64[2], xyz_min[2])}, p1[3] = {x1, y1, z1};
                lerp3_64(p0, p1, sample(&g, x + 1, y + 1, z), v6, iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
            if (r->info & 2u) {
                double p0[3] = {x1, ijk_to_xyz64(y, csz[1], rng64[1], xyz_min[1]), z1}, p1[3] = {x1, y1, z1};
                lerp3_64(p0, p1, sample(&g, x + 1, y, z + 1), v6, iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
            if (r->info & 4u) {
                double p0[3] = {x1, y1, z1}, p1[3] = {ijk_to_xyz64(x, csz[0], rng64[0], xyz_min[0]), y1, z1};
                lerp3_64(p0, p1, v6, sample(&g, x, y + 1, z + 1), iso, &vt[3 * (uint64_t)vi]); ++vi;
            }
        }
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            int64_t x = (int64_t)(i1 % g.cx), y = (int64_t)((i1 / g.cx) % g.cy), z = (int64_t)(i1 / (g.cx * g.cy));
            uint8_t cnt[4] = {0, 0, 0, 0};
            double acc[4][3] = {{0}};
            for (int e = 0; e < 12; ++e) {
                uint8_t m = lut_m(r, e);
                if (m == 0xff) continue;
                int64_t ox = x + OWNER_OFF[e][0], oy = y + OWNER_OFF[e][1], oz = z + OWNER_OFF[e][2];
                if (ox < 0 || oy < 0 || oz < 0) continue;
                uint64_t oi = ((uint64_t)oz * g.cy + (uint64_t)oy) * g.cx + (uint64_t)ox;
                const cell_rec *owner = &rec[map[oi]];
                const double *src = &vt[3 * (uint64_t)edge_vertex_index(owner, OWNER_EDGE[e])];
                acc[m][0] += src[0]; acc[m][1] += src[1]; acc[m][2] += src[2];
                cnt[m]++;
            }
            uint8_t niso = (uint8_t)(r->nv - ((r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u)));
            for (uint8_t m = 0; m < niso; ++m) {
                double *dst = &vt[3 * ((uint64_t)r->vertex_begin + m)];
                if (!cnt[m]) {
                    for (int e = 0; e < 12; ++e) {
                        if (lut_m(r, e) != m) continue;
                        double c3[3];
                        crossing_local64(&g, (uint64_t)x, (uint64_t)y, (uint64_t)z, e, iso, rng64, xyz_min, csz, c3);
                        acc[m][0] += c3[0]; acc[m][1] += c3[1]; acc[m][2] += c3[2];
                        cnt[m]++;
                    }
                }
                dst[0] = acc[m][0] / cnt[m]; dst[1] = acc[m][1] / cnt[m]; dst[2] = acc[m][2] / cnt[m];
            }
        }
    }

    /* step 7: quads (dmc.cu:1983-2047).  Count per cell, exclusive scan, fill. */
    uint32_t *qoff = (uint32_t *)malloc((A ? A : 1) * sizeof(uint32_t));
    if (!qoff) { free(aoff); free(map); free(cfg); free(rec); return 2; }
    /* quads per owner cell (into qoff for now), then the blocked scan */
    uint64_t dropped = 0;
    #pragma omp parallel for reduction(+:dropped) schedule(static)
    for (int64_t a = 0; a < (int64_t)A; ++a) {
        const cell_rec *r = &rec[a];
        uint64_t i1 = r->index1d;
        uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
        static const int P0[3] = {2, 5, 7};
        uint32_t nq = 0;
        for (int s = 0; s < 3; ++s) {
            if (!((r->info >> s) & 1u)) continue;
            int exceed = s == 0 ? (x + 1 >= g.cx || y + 1 >= g.cy)
                       : s == 1 ? (x + 1 >= g.cx || z + 1 >= g.cz)
                                : (y + 1 >= g.cy || z + 1 >= g.cz);
            if (exceed) continue;
            if (((r->config >> P0[s]) & 1u) == ((r->config >> 6) & 1u)) { dropped++; continue; }
            nq++;
        }
        qoff[a] = nq;
    }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk_a; ++b) {
        const uint64_t a0 = (uint64_t)b * SCAN_BLOCK, a1 = a0 + SCAN_BLOCK < A ? a0 + SCAN_BLOCK : A;
        uint64_t n = 0;
        for (uint64_t a = a0; a < a1; ++a) n += qoff[a];
        aoff[b + 1] = n;
    }
    aoff[0] = 0;
    for (uint64_t b = 0; b < nblk_a; ++b) aoff[b + 1] += aoff[b];
    const uint64_t Q = aoff[nblk_a];
    out->n_dropped_quads = dropped;
    if (Q >= INVALID32) { free(aoff); free(map); free(cfg); free(rec); free(qoff); return 3; }
    #pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < (int64_t)nblk_a; ++b) {
        const uint64_t a0 = (uint64_t)b * SCAN_BLOCK, a1 = a0 + SCAN_BLOCK < A ? a0 + SCAN_BLOCK : A;
        uint64_t q = aoff[b];
        for (uint64_t a = a0; a < a1; ++a) { const uint32_t n = qoff[a]; qoff[a] = (uint32_t)q; q += n; }
    }
    free(aoff);
    out->n_quads = Q;
    uint32_t *qd = (uint32_t *)malloc((Q ? Q : 1) * 4 * sizeof(uint32_t));
    if (!qd) { free(map); free(cfg); free(rec); free(qoff); return 2; }
    out->quads = qd;
    #pragma omp parallel for schedule(static)
    for (int64_t a = 0; a < (int64_t)A; ++a) {
        const cell_rec *r = &rec[a];
        uint64_t i1 = r->index1d;
        uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
        uint64_t q = qoff[a];
        static const int P0[3] = {2, 5, 7};
        for (int s = 0; s < 3; ++s) {
            if (!((r->info >> s) & 1u)) continue;
            int exceed = s == 0 ? (x + 1 >= g.cx || y + 1 >= g.cy)
                       : s == 1 ? (x + 1 >= g.cx || z + 1 >= g.cz)
                                : (y + 1 >= g.cy || z + 1 >= g.cz);
            if (exceed) continue;
            if (((r->config >> P0[s]) & 1u) == ((r->config >> 6) & 1u)) continue;
            int ccw = (r->info >> (s + 3)) & 1u;
            /* CircularEdgeRange (dmc.cu:1595-1691): ccw visits 0,1,2,3; cw 0,3,2,1.
             * Ring cell for ring edge re sits at -OWNER_OFF[re] from this cell. */
            for (int it = 0; it < 4; ++it) {
                int k = ccw ? it : (4 - it) % 4;
                int re = RING[s][k];
                uint64_t rx = x - OWNER_OFF[re][0], ry = y - OWNER_OFF[re][1], rz = z - OWNER_OFF[re][2];
                uint64_t ri = (rz * g.cy + ry) * g.cx + rx;
                const cell_rec *rr = &rec[map[ri]];
                qd[4 * q + it] = rr->vertex_begin + lut_m(rr, re);
            }
            ++q;
        }
    }

    /* step 8: smoothing iterations (dmc.cu:2157-2169) */
    float *vt = out->vertices;
    for (uint32_t it = 0; it < num_smooth; ++it) {
        /* smooth_edge_vertices: reads dual vertices, writes crossings */
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            const cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            uint64_t x = i1 % g.cx, y = (i1 / g.cx) % g.cy, z = i1 / (g.cx * g.cy);
            uint64_t q = qoff[a];
            static const int P0[3] = {2, 5, 7};
            static const int EDGE[3] = {6, 9, 10};
            for (int s = 0; s < 3; ++s) {
                if (!((r->info >> s) & 1u)) continue;
                int exceed = s == 0 ? (x + 1 >= g.cx || y + 1 >= g.cy)
                           : s == 1 ? (x + 1 >= g.cx || z + 1 >= g.cz)
                                    : (y + 1 >= g.cy || z + 1 >= g.cz);
                if (exceed) continue;
                if (((r->config >> P0[s]) & 1u) == ((r->config >> 6) & 1u)) continue;
                const float x1 = ijk_to_xyz(x + 1, csz[0], rng[0], xyz_min[0]);
                const float y1 = ijk_to_xyz(y + 1, csz[1], rng[1], xyz_min[1]);
                const float z1 = ijk_to_xyz(z + 1, csz[2], rng[2], xyz_min[2]);
                const float origin[2] = {s == 2 ? y1 : x1, s == 0 ? y1 : z1};
                float nv3[3];
                if (smooth_edge(vt, &qd[4 * q], s, origin, nv3)) {
                    float *dst = &vt[3 * (uint64_t)edge_vertex_index(r, EDGE[s])];
                    dst[0] = nv3[0]; dst[1] = nv3[1]; dst[2] = nv3[2];
                }
                ++q;
            }
        }
        /* calc_iso_vertices_kern: dual vertices from the current crossings;
         * a patch without an owner inside the volume keeps its position */
        #pragma omp parallel for schedule(static)
        for (int64_t a = 0; a < (int64_t)A; ++a) {
            cell_rec *r = &rec[a];
            uint64_t i1 = r->index1d;
            int64_t x = (int64_t)(i1 % g.cx), y = (int64_t)((i1 / g.cx) % g.cy), z = (int64_t)(i1 / (g.cx * g.cy));
            uint8_t cnt[4] = {0, 0, 0, 0};
            float acc[4][3];
            for (int e = 0; e < 12; ++e) {
                uint8_t m = lut_m(r, e);
                if (m == 0xff) continue;
                int64_t ox = x + OWNER_OFF[e][0], oy = y + OWNER_OFF[e][1], oz = z + OWNER_OFF[e][2];
                if (ox < 0 || oy < 0 || oz < 0) continue;
                uint64_t oi = ((uint64_t)oz * g.cy + (uint64_t)oy) * g.cx + (uint64_t)ox;
                const float *src = &vt[3 * (uint64_t)edge_vertex_index(&rec[map[oi]], OWNER_EDGE[e])];
                if (cnt[m] == 0) { acc[m][0] = src[0]; acc[m][1] = src[1]; acc[m][2] = src[2]; }
                else { acc[m][0] = acc[m][0] + src[0]; acc[m][1] = acc[m][1] + src[1]; acc[m][2] = acc[m][2] + src[2]; }
                cnt[m]++;
            }
            uint8_t niso = (uint8_t)(r->nv - ((r->info & 1u) + ((r->info >> 1) & 1u) + ((r->info >> 2) & 1u)));
            for (uint8_t m = 0; m < niso; ++m) {
                if (!cnt[m]) continue;
                float d = (float)cnt[m];
                float *dst = &vt[3 * ((uint64_t)r->vertex_begin + m)];
                dst[0] = acc[m][0] / d; dst[1] = acc[m][1] / d; dst[2] = acc[m][2] / d;
            }
        }
    }
    free(qoff); free(map); free(cfg); free(rec);
    return 0;
}
