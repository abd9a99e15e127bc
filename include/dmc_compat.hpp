// dmc_compat.hpp — the reference's C++ call shape on top of the C ABI.
//
// A caller of the reference (vcg-thin-meshgen/Framework,
// DMC_CUDA/DMC_CUDA/include/dmc.hpp:40-57) includes this header instead of
// dmc.hpp and keeps its calls:
//
//     dmc::setup_device_luts();                                   // dmc.hpp:40
//     dmc::run_dmc(vertices, triangles, grid, xyz_min, xyz_max,   // dmc.hpp:56-57
//                  iso_value, num_smooth);
//     dmc::cleanup_device_luts();                                 // dmc.hpp:48
//
// `grid` may be the reference's utils::Array3D<float> or anything else with
// dim_x(), dim_y(), dim_z() and a contiguous x-fastest data() of float (or
// uint16_t).  Vertices and triangles come back in the reference's order and
// split.  Where the reference prints and calls exit(1) on an error
// (cuda_includes.h:13-19), these calls throw dmc::error carrying the status.
// dump_obj mirrors the reference's helper (dmc.cu:2238-2246).
//
// The context is process-wide, like the reference's device tables, and the
// calls are not thread-safe (neither are the reference's); threaded callers
// use the C ABI with one dmc_ctx per thread.
#pragma once
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>
#include <vector_types.h>   // float3, uint3
#include "dmc_gb300.h"

namespace dmc {

class error : public std::runtime_error {
public:
    error(dmc_status s, const char *what)
        : std::runtime_error(std::string(what) + ": " + dmc_status_string(s)), status(s) {}
    dmc_status status;
};

namespace detail {
inline dmc_ctx *&context()
{
    static dmc_ctx *ctx = nullptr;
    return ctx;
}
inline void check(dmc_status s, const char *what)
{
    if (s != DMC_OK) throw error(s, what);
}
}  // namespace detail

inline void setup_device_luts(int device = 0)
{
    if (!detail::context()) detail::check(dmc_create(&detail::context(), device), "dmc::setup_device_luts");
}

inline void cleanup_device_luts()
{
    if (detail::context()) {
        dmc_destroy(detail::context());
        detail::context() = nullptr;
    }
}

template <class Grid>
void run_dmc(std::vector<float3> &vertices, std::vector<uint3> &triangles, const Grid &grid, const float3 &xyz_min,
             const float3 &xyz_max, float iso_value, unsigned num_smooth = 0)
{
    using T = typename std::remove_cv<typename std::remove_pointer<decltype(grid.data())>::type>::type;
    static_assert(std::is_same<T, float>::value || std::is_same<T, uint16_t>::value,
                  "grid samples must be float or uint16_t");
    setup_device_luts();
    dmc_volume vol;
    vol.data = grid.data();
    vol.dtype = std::is_same<T, float>::value ? DMC_F32 : DMC_U16;
    vol.dims[0] = grid.dim_x();
    vol.dims[1] = grid.dim_y();
    vol.dims[2] = grid.dim_z();
    const float mn[3] = {xyz_min.x, xyz_min.y, xyz_min.z};
    const float mx[3] = {xyz_max.x, xyz_max.y, xyz_max.z};
    dmc_mesh m{};
    detail::check(dmc_run(detail::context(), &vol, mn, mx, iso_value, num_smooth, 1, &m), "dmc::run_dmc");
    const float3 *v = reinterpret_cast<const float3 *>(m.vertices);
    const uint3 *t = reinterpret_cast<const uint3 *>(m.triangles);
    vertices.assign(v, v + m.n_vertices);
    triangles.assign(t, t + m.n_triangles);
    dmc_mesh_free(&m);
}

inline void dump_obj(const char *filename, const std::vector<float3> &vertices, const std::vector<uint3> &triangles)
{
    detail::check(dmc_write_obj(filename, reinterpret_cast<const float *>(vertices.data()), vertices.size(),
                                reinterpret_cast<const uint32_t *>(triangles.data()), triangles.size(), 3),
                  "dmc::dump_obj");
}

}  // namespace dmc
