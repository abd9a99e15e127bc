// Mesh file output (host only): Wavefront OBJ in the reference's format
// (dump_obj, dmc.cu:2238-2246): one "v x y z" line per vertex with the
// default six significant digits of a C++ stream (printf %g), then one
// "f a b c" (or "f a b c d") line per face with 1-based indices.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include "../../include/dmc_gb300.h"

extern "C" dmc_status dmc_write_obj(const char *path, const float *vertices, uint64_t n_vertices,
                                    const uint32_t *faces, uint64_t n_faces, uint32_t verts_per_face)
{
    if (!path || (n_vertices && !vertices) || (n_faces && !faces)) return DMC_ERR_INVALID_ARG;
    if (verts_per_face != 3 && verts_per_face != 4) return DMC_ERR_INVALID_ARG;
    for (uint64_t i = 0; i < n_faces * verts_per_face; ++i)
        if (faces[i] >= n_vertices) return DMC_ERR_INVALID_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return DMC_ERR_INVALID_ARG;
    const size_t cap = 1 << 22;
    char *buf = (char *)malloc(cap + 256);
    if (!buf) { fclose(f); return DMC_ERR_OOM; }
    size_t len = 0;
    bool ok = true;
    auto flush = [&](bool force) {
        if (len && (force || len >= cap)) {
            ok = ok && fwrite(buf, 1, len, f) == len;
            len = 0;
        }
    };
    for (uint64_t i = 0; i < n_vertices; ++i) {
        len += (size_t)snprintf(buf + len, 256, "v %g %g %g\n", (double)vertices[3 * i], (double)vertices[3 * i + 1],
                                (double)vertices[3 * i + 2]);
        flush(false);
    }
    for (uint64_t i = 0; i < n_faces; ++i) {
        const uint32_t *t = faces + (size_t)verts_per_face * i;
        if (verts_per_face == 3)
            len += (size_t)snprintf(buf + len, 256, "f %u %u %u\n", t[0] + 1, t[1] + 1, t[2] + 1);
        else
            len += (size_t)snprintf(buf + len, 256, "f %u %u %u %u\n", t[0] + 1, t[1] + 1, t[2] + 1, t[3] + 1);
        flush(false);
    }
    flush(true);
    free(buf);
    ok = (fclose(f) == 0) && ok;
    return ok ? DMC_OK : DMC_ERR_INVALID_ARG;
}
