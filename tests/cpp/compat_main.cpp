// Drives include/dmc_compat.hpp the way a caller of the reference would:
// an Array3D-like grid of a sampled sphere, dmc::run_dmc, dmc::dump_obj.
// Usage: compat_main <n> <iso> <out.obj>   (prints "V T" on success,
// "error <status>" when the library reports an error, e.g. without a GPU)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <vector_functions.h>   // make_float3
#include "dmc_compat.hpp"

struct Grid {   // the reference's utils::Array3D interface (utils.hpp:15-66)
    unsigned nx, ny, nz;
    std::vector<float> v;
    unsigned dim_x() const { return nx; }
    unsigned dim_y() const { return ny; }
    unsigned dim_z() const { return nz; }
    const float *data() const { return v.data(); }
};

int main(int argc, char **argv)
{
    const unsigned n = argc > 1 ? (unsigned)atoi(argv[1]) : 21;
    const float iso = argc > 2 ? (float)atof(argv[2]) : 4.1f;
    Grid g{n, n, n, std::vector<float>((size_t)n * n * n)};
    const float lo = -5.f, range = 10.f;
    for (unsigned k = 0; k < n; ++k)
        for (unsigned j = 0; j < n; ++j)
            for (unsigned i = 0; i < n; ++i) {
                float x = (float)i / (n - 1) * range + lo, y = (float)j / (n - 1) * range + lo, z = (float)k / (n - 1) * range + lo;
                g.v[((size_t)k * n + j) * n + i] = std::sqrt(x * x + y * y + z * z);
            }
    std::vector<float3> verts;
    std::vector<uint3> tris;
    try {
        dmc::setup_device_luts();
        dmc::run_dmc(verts, tris, g, make_float3(lo, lo, lo), make_float3(lo + range, lo + range, lo + range), iso, 0);
        if (argc > 3) dmc::dump_obj(argv[3], verts, tris);
        dmc::cleanup_device_luts();
    } catch (const dmc::error &e) {
        std::printf("error %d\n", (int)e.status);
        return 0;
    }
    std::printf("%zu %zu\n", verts.size(), tris.size());
    return 0;
}
