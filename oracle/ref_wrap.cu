// C entry points over the reference's own dmc::run_dmc (DMC_CUDA/DMC_CUDA/
// include/dmc.hpp:40-57), for tests/golden/make_ref_golden.py: it loads the
// library that oracle/build_ref.py builds from the unmodified reference
// sources.  Test infrastructure only.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dmc.hpp"

extern "C" {

// Runs the reference on a float volume (x fastest, dims = points per axis).
// The reference's errors end the process (cuda_includes.h:13-19).  Returns
// malloc'd vertex (3 floats each) and triangle (3 uint32 each) arrays.
int dmcref_run(const float *grid, const unsigned dims[3], const float mn[3], const float mx[3], float iso,
               unsigned num_smooth, float **verts, uint64_t *n_verts, unsigned **tris, uint64_t *n_tris)
{
    utils::Array3D<float> g(dims[0], dims[1], dims[2]);
    std::memcpy(g.data(), grid, sizeof(float) * g.size());
    std::vector<float3> v;
    std::vector<uint3> t;
    dmc::run_dmc(v, t, g, make_float3(mn[0], mn[1], mn[2]), make_float3(mx[0], mx[1], mx[2]), iso, num_smooth);
    *n_verts = v.size();
    *n_tris = t.size();
    *verts = (float *)std::malloc(sizeof(float) * 3 * (v.size() ? v.size() : 1));
    *tris = (unsigned *)std::malloc(sizeof(unsigned) * 3 * (t.size() ? t.size() : 1));
    if (!*verts || !*tris) return 1;
    for (size_t i = 0; i < v.size(); ++i) {
        (*verts)[3 * i] = v[i].x; (*verts)[3 * i + 1] = v[i].y; (*verts)[3 * i + 2] = v[i].z;
    }
    for (size_t i = 0; i < t.size(); ++i) {
        (*tris)[3 * i] = t[i].x; (*tris)[3 * i + 1] = t[i].y; (*tris)[3 * i + 2] = t[i].z;
    }
    return 0;
}

void dmcref_setup(void) { dmc::setup_device_luts(); }
void dmcref_cleanup(void) { dmc::cleanup_device_luts(); }
void dmcref_free(void *p) { std::free(p); }

}
