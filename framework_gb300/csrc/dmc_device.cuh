// Device-side building blocks shared by every extraction kernel.
//
// Arithmetic contract (bit-exact with the reference's FP32 path): every float
// operation below is an explicitly rounded intrinsic (__fadd_rn, __fmul_rn,
// __fdiv_rn), so the compiler cannot fuse a multiply and an add.  The order of
// operations follows the reference:
//   ijk_to_xyz  utils.hpp:118-122   (float)i / size * range + min
//   lerp_float3 dmc.cu:1090-1098    t=(iso-v0)/(v1-v0); p0*(1-t) + p1*t
//   dual vertex dmc.cu:1517-1593    crossings summed in edge order 0..11
//                                   (first assigned, then added), / count
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace dmc {

#include "dmc_tables.inc"

// Tables on the device (one copy per context in global memory; the brick
// kernels stage it in shared memory).  Lookups happen only for active cells.
struct DeviceTables {
    uint8_t edge_lut[2][256 * 12];   // dual vertex of a cell per edge; 0xff = none
    uint8_t nvert[2][256];           // dual vertices per config
    uint8_t amb_face[256];           // ambiguous face of a 2B/3B config, 0xff otherwise
    uint8_t face_dir[8];             // neighbour direction of a face: 0 +x,1 -x,2 +y,3 -y,4 +z,5 -z
    uint16_t crossed[256];           // bit e: edge e changes sign under this config
};

// Owner of each cell edge: offset (0 or -1 per axis) to the cell that owns it
// and that cell's edge (6 = z, 9 = y, 10 = x), dmc.cu:634-649.
__device__ __forceinline__ int owner_dx(int e) { return (e == 3 || e == 4 || e == 7 || e == 11) ? -1 : 0; }
__device__ __forceinline__ int owner_dy(int e) { return (e == 0 || e == 4 || e == 5 || e == 8) ? -1 : 0; }
__device__ __forceinline__ int owner_dz(int e) { return (e == 0 || e == 1 || e == 2 || e == 3) ? -1 : 0; }

template <class T> __device__ __forceinline__ float load_sample(const T *p, uint64_t i);
template <> __device__ __forceinline__ float load_sample<float>(const float *p, uint64_t i) { return __ldg(p + i); }
template <> __device__ __forceinline__ float load_sample<uint16_t>(const uint16_t *p, uint64_t i)
{
    return __uint2float_rn((unsigned)__ldg(p + i));
}

__device__ __forceinline__ float ijk_to_xyz(uint32_t i, uint32_t size, float range, float mn)
{
    return __fadd_rn(__fmul_rn(__fdiv_rn(__uint2float_rn(i), __uint2float_rn(size)), range), mn);
}

struct Geo {
    float x0, x1, y0, y1, z0, z1;   // world coordinates of the cell's two planes per axis
};

__device__ __forceinline__ Geo cell_geo(uint32_t x, uint32_t y, uint32_t z, uint3 cells, float3 rng, float3 mn)
{
    Geo g;
    g.x0 = ijk_to_xyz(x, cells.x, rng.x, mn.x); g.x1 = ijk_to_xyz(x + 1, cells.x, rng.x, mn.x);
    g.y0 = ijk_to_xyz(y, cells.y, rng.y, mn.y); g.y1 = ijk_to_xyz(y + 1, cells.y, rng.y, mn.y);
    g.z0 = ijk_to_xyz(z, cells.z, rng.z, mn.z); g.z1 = ijk_to_xyz(z + 1, cells.z, rng.z, mn.z);
    return g;
}

__device__ __forceinline__ float3 lerp3(float ax, float ay, float az, float bx, float by, float bz,
                                        float v0, float v1, float iso)
{
    float t = __fdiv_rn(__fsub_rn(iso, v0), __fsub_rn(v1, v0));
    float omt = __fsub_rn(1.0f, t);
    float3 r;
    r.x = __fadd_rn(__fmul_rn(ax, omt), __fmul_rn(bx, t));
    r.y = __fadd_rn(__fmul_rn(ay, omt), __fmul_rn(by, t));
    r.z = __fadd_rn(__fmul_rn(az, omt), __fmul_rn(bz, t));
    return r;
}

// Crossing of edge e of a cell, evaluated in the orientation of the edge's
// owner (edge 6: low z -> high z, dmc.cu:1490; edge 9: low y -> high y,
// :1500; edge 10: high x -> low x, :1509), so that it equals the owner's
// emitted edge vertex bit for bit.  v[] are the cell's corner samples.
__device__ __forceinline__ float3 edge_crossing(int e, const float v[8], const Geo &g, float iso)
{
    switch (e) {
    // x edges: from the high-x corner to the low-x corner
    case 0:  return lerp3(g.x1, g.y0, g.z0, g.x0, g.y0, g.z0, v[1], v[0], iso);
    case 2:  return lerp3(g.x1, g.y1, g.z0, g.x0, g.y1, g.z0, v[2], v[3], iso);
    case 8:  return lerp3(g.x1, g.y0, g.z1, g.x0, g.y0, g.z1, v[5], v[4], iso);
    case 10: return lerp3(g.x1, g.y1, g.z1, g.x0, g.y1, g.z1, v[6], v[7], iso);
    // y edges: low y to high y
    case 1:  return lerp3(g.x1, g.y0, g.z0, g.x1, g.y1, g.z0, v[1], v[2], iso);
    case 3:  return lerp3(g.x0, g.y0, g.z0, g.x0, g.y1, g.z0, v[0], v[3], iso);
    case 9:  return lerp3(g.x1, g.y0, g.z1, g.x1, g.y1, g.z1, v[5], v[6], iso);
    case 11: return lerp3(g.x0, g.y0, g.z1, g.x0, g.y1, g.z1, v[4], v[7], iso);
    // z edges: low z to high z
    case 4:  return lerp3(g.x0, g.y0, g.z0, g.x0, g.y0, g.z1, v[0], v[4], iso);
    case 5:  return lerp3(g.x1, g.y0, g.z0, g.x1, g.y0, g.z1, v[1], v[5], iso);
    case 6:  return lerp3(g.x1, g.y1, g.z0, g.x1, g.y1, g.z1, v[2], v[6], iso);
    default: return lerp3(g.x0, g.y1, g.z0, g.x0, g.y1, g.z1, v[3], v[7], iso);
    }
}

// dmc.cu:1018-1027: bit i set when corner i is below the isovalue.
__device__ __forceinline__ uint32_t config_of(const float v[8], float iso)
{
    uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) m |= (v[i] < iso ? 1u : 0u) << i;
    return m;
}

// dmc.cu:1101-1106 (reference bipolarity of an edge, including the case where
// one sample equals the isovalue and the other is above it).
__device__ __forceinline__ bool ref_bipolar(float a, float b, float iso)
{
    if (a == b) return false;
    float lo = a > b ? b : a, hi = a > b ? a : b;
    return !((lo < iso && hi < iso) || (lo > iso && hi > iso));
}

// Owned-edge info of a cell (dmc.cu:1173-1221): bits 0-2 = edges 6, 9, 10
// bipolar (reference test), bits 3-5 = ccw (v[p0] <= iso, p0 = 2, 5, 7).
__device__ __forceinline__ uint32_t owned_edge_info(const float v[8], float iso)
{
    uint32_t info = 0;
    if (ref_bipolar(v[2], v[6], iso)) info |= 1u | (v[2] <= iso ? 8u : 0u);
    if (ref_bipolar(v[5], v[6], iso)) info |= 2u | (v[5] <= iso ? 16u : 0u);
    if (ref_bipolar(v[7], v[6], iso)) info |= 4u | (v[7] <= iso ? 32u : 0u);
    return info;
}

// Owned edge s (0: edge 6, 1: edge 9, 2: edge 10) changes sign in the config
// bits: corners (2,6), (5,6), (7,6).
__device__ __forceinline__ bool owned_sign_change(uint32_t cfg, int s)
{
    int p0 = s == 0 ? 2 : (s == 1 ? 5 : 7);
    return ((cfg >> p0) & 1u) != ((cfg >> 6) & 1u);
}

// Quad around owned edge s of cell (x,y,z) lies inside the volume
// (circular_edge_exceed_boundary, dmc.cu:1696-1708).
__device__ __forceinline__ bool owned_quad_in_volume(int s, uint32_t x, uint32_t y, uint32_t z, uint3 cells)
{
    if (s == 0) return x + 1 < cells.x && y + 1 < cells.y;
    if (s == 1) return x + 1 < cells.x && z + 1 < cells.z;
    return y + 1 < cells.y && z + 1 < cells.z;
}

// Ring of cells around owned edge s in ccw order (circular_edge_lut,
// dmc.cu:653-658, offsets negated as in dmc.cu:1656-1664): the edge in the
// ring cell and the ring cell's offset from the owner.
__device__ __forceinline__ void ring_entry(int s, int k, int &edge, int &dx, int &dy, int &dz)
{
    // s=0: 6,7,4,5   s=1: 9,1,3,11   s=2: 10,8,0,2
    const int E[3][4] = {{6, 7, 4, 5}, {9, 1, 3, 11}, {10, 8, 0, 2}};
    edge = E[s][k];
    dx = -owner_dx(edge); dy = -owner_dy(edge); dz = -owner_dz(edge);
}

__device__ __forceinline__ uint32_t nvert_of(const DeviceTables &tab, uint32_t cfg, bool lut2)
{
    return tab.nvert[lut2 ? 1 : 0][cfg];
}
__device__ __forceinline__ uint32_t lut_m(const DeviceTables &tab, uint32_t cfg, bool lut2, int e)
{
    return tab.edge_lut[lut2 ? 1 : 0][cfg * 12 + e];
}

// Dual vertices of an active cell: writes niso float3 at out[0..niso).
// Crossings of edges whose owner lies below the volume are left out, as the
// reference does (dmc.cu:1556-1562).  A dual vertex whose patch has no edge
// with an owner inside the volume is never written by the reference (it is
// unreferenced); here it gets the mean of its patch's crossings.
__device__ __forceinline__ void dual_vertices(const DeviceTables &tab, const float v[8], const Geo &g, float iso, uint32_t cfg, bool lut2,
                                              uint32_t x, uint32_t y, uint32_t z, uint32_t niso, float *out)
{
    float3 acc[4];
    uint32_t cnt[4] = {0, 0, 0, 0};
    acc[0] = acc[1] = acc[2] = acc[3] = make_float3(0.f, 0.f, 0.f);
#pragma unroll
    for (int e = 0; e < 12; ++e) {
        uint32_t m = lut_m(tab, cfg, lut2, e);
        if (m == 0xffu) continue;
        if ((owner_dx(e) < 0 && x == 0) || (owner_dy(e) < 0 && y == 0) || (owner_dz(e) < 0 && z == 0)) continue;
        float3 c = edge_crossing(e, v, g, iso);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (m == (uint32_t)k) {
                if (cnt[k] == 0) acc[k] = c;
                else { acc[k].x = __fadd_rn(acc[k].x, c.x); acc[k].y = __fadd_rn(acc[k].y, c.y); acc[k].z = __fadd_rn(acc[k].z, c.z); }
                cnt[k]++;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if ((uint32_t)k >= niso) break;
        if (cnt[k] == 0) {
            for (int e = 0; e < 12; ++e) {
                if (lut_m(tab, cfg, lut2, e) != (uint32_t)k) continue;
                float3 c = edge_crossing(e, v, g, iso);
                if (cnt[k] == 0) acc[k] = c;
                else { acc[k].x = __fadd_rn(acc[k].x, c.x); acc[k].y = __fadd_rn(acc[k].y, c.y); acc[k].z = __fadd_rn(acc[k].z, c.z); }
                cnt[k]++;
            }
        }
        float d = __uint2float_rn(cnt[k]);
        out[3 * k + 0] = __fdiv_rn(acc[k].x, d);
        out[3 * k + 1] = __fdiv_rn(acc[k].y, d);
        out[3 * k + 2] = __fdiv_rn(acc[k].z, d);
    }
}

// Edge vertices of the cell's own edges 6, 9, 10 that are bipolar by the
// reference's test, in that order (dmc.cu:1468-1514).
__device__ __forceinline__ void owned_edge_vertices(const float v[8], const Geo &g, float iso, uint32_t info, float *out)
{
    int n = 0;
    if (info & 1u) { float3 c = edge_crossing(6, v, g, iso);  out[3*n] = c.x; out[3*n+1] = c.y; out[3*n+2] = c.z; ++n; }
    if (info & 2u) { float3 c = edge_crossing(9, v, g, iso);  out[3*n] = c.x; out[3*n+1] = c.y; out[3*n+2] = c.z; ++n; }
    if (info & 4u) { float3 c = edge_crossing(10, v, g, iso); out[3*n] = c.x; out[3*n+1] = c.y; out[3*n+2] = c.z; ++n; }
}

// Corners of each edge in the order its owner evaluates the crossing
// (owner edge 6: low z to high z; 9: low y to high y; 10: high x to low x),
// 4 bits per edge, edge 0 in the lowest nibble.
constexpr unsigned long long kEdgeFrom = 0x465532100211ull;
constexpr unsigned long long kEdgeTo = 0x776476543320ull;

__device__ __forceinline__ float pick8(const float v[8], int c)
{
    const float s01 = (c & 1) ? v[1] : v[0], s23 = (c & 1) ? v[3] : v[2];
    const float s45 = (c & 1) ? v[5] : v[4], s67 = (c & 1) ? v[7] : v[6];
    const float t0 = (c & 2) ? s23 : s01, t1 = (c & 2) ? s67 : s45;
    return (c & 4) ? t1 : t0;
}

// edge_crossing for a run-time edge index, without a per-edge branch.
__device__ __forceinline__ float3 crossing_any(int e, const float v[8], const Geo &g, float iso)
{
    const int a = (int)((kEdgeFrom >> (4 * e)) & 15ull), b = (int)((kEdgeTo >> (4 * e)) & 15ull);
    // corner c sits at x = (c ^ c >> 1) & 1, y = c >> 1 & 1, z = c >> 2
    const float ax = ((a ^ (a >> 1)) & 1) ? g.x1 : g.x0, ay = ((a >> 1) & 1) ? g.y1 : g.y0, az = (a >> 2) ? g.z1 : g.z0;
    const float bx = ((b ^ (b >> 1)) & 1) ? g.x1 : g.x0, by = ((b >> 1) & 1) ? g.y1 : g.y0, bz = (b >> 2) ? g.z1 : g.z0;
    return lerp3(ax, ay, az, bx, by, bz, pick8(v, a), pick8(v, b), iso);
}

__device__ __forceinline__ float3 add3(float3 a, float3 b)
{
    return make_float3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}

// acc / n as the reference computes it (a true IEEE division); division by a
// power of two is the exact multiplication by its reciprocal, so it is used
// for n = 1, 2, 4, 8 (same rounded result).
__device__ __forceinline__ float3 div3(float3 a, uint32_t n)
{
    if (n == 1 || n == 2 || n == 4 || n == 8) {
        const float r = n == 1 ? 1.f : (n == 2 ? 0.5f : (n == 4 ? 0.25f : 0.125f));
        return make_float3(__fmul_rn(a.x, r), __fmul_rn(a.y, r), __fmul_rn(a.z, r));
    }
    const float d = __uint2float_rn(n);
    float c[3] = {a.x, a.y, a.z};
#pragma unroll 1
    for (int i = 0; i < 3; ++i) c[i] = __fdiv_rn(c[i], d);
    return make_float3(c[0], c[1], c[2]);
}

__device__ __forceinline__ void store3(float *p, float3 c) { p[0] = c.x; p[1] = c.y; p[2] = c.z; }

// Dual vertices of a cell with several patches (rare): crossings of the
// owner-inside edges accumulated per patch in edge order; a patch with none
// of them takes all its crossings.
struct Corners { float v[8]; };

static __device__ __noinline__ void multi_patch_vertices(const DeviceTables &tab, const Corners cv, Geo g, float iso,
                                                         uint32_t cfg, bool lut2, uint32_t niso, uint32_t cm, uint32_t om,
                                                         float *out)
{
    const float *v = cv.v;
    float3 acc[4];
    uint32_t cnt[4] = {0, 0, 0, 0};
    uint32_t mm = om;
    while (mm) {
        const int e = __ffs(mm) - 1;
        mm &= mm - 1;
        const float3 c = crossing_any(e, v, g, iso);
        const uint32_t m = lut_m(tab, cfg, lut2, e);
        acc[m] = cnt[m] ? add3(acc[m], c) : c;
        cnt[m]++;
    }
    for (uint32_t m = 0; m < niso; ++m) {
        if (cnt[m] == 0) {
            uint32_t fm = cm;
            while (fm) {
                const int e = __ffs(fm) - 1;
                fm &= fm - 1;
                if (lut_m(tab, cfg, lut2, e) != m) continue;
                const float3 c = crossing_any(e, v, g, iso);
                acc[m] = cnt[m] ? add3(acc[m], c) : c;
                cnt[m]++;
            }
        }
        store3(out + 3 * m, div3(acc[m], cnt[m]));
    }
}

// All vertices of an active cell, written to out: the niso dual vertices,
// then the crossings of its own edges 6, 9, 10 flagged in info (bits 0-2).
// Same values as dual_vertices + owned_edge_vertices; each needed crossing
// is evaluated once, at a single call site (keeps the kernel small).
__device__ __forceinline__ void cell_vertices(const DeviceTables &tab, const float v[8], const Geo &g, float iso,
                                              uint32_t cfg, bool lut2, uint32_t niso, uint32_t info,
                                              uint32_t x, uint32_t y, uint32_t z, float *out)
{
    const uint32_t cm = tab.crossed[cfg];
    uint32_t om = cm;                      // crossed edges whose owner lies inside the volume
    if (x == 0) om &= ~0x898u;             // edges 3, 4, 7, 11 are owned at -x
    if (y == 0) om &= ~0x131u;             // edges 0, 4, 5, 8 are owned at -y
    if (z == 0) om &= ~0x00fu;             // edges 0, 1, 2, 3 are owned at -z
    // edges of the single patch that enter the mean, and owned edges whose
    // crossing is emitted
    const uint32_t dual = niso == 1 ? (om ? om : cm) : 0u;
    const uint32_t owned = ((info & 1u) << 6) | ((info & 2u) << 8) | ((info & 4u) << 8);
    // an owned crossing goes out as soon as it is evaluated: after the niso
    // dual vertices, in the order 6, 9, 10 (the order of the bits)
    float *const own_out = out + 3 * niso;
    float3 acc = make_float3(0.f, 0.f, 0.f);
    uint32_t n = 0, mm = dual | owned;
    while (mm) {
        const int e = __ffs(mm) - 1;
        mm &= mm - 1;
        const float3 c = crossing_any(e, v, g, iso);
        if ((dual >> e) & 1u) { acc = n ? add3(acc, c) : c; ++n; }
        if ((owned >> e) & 1u) store3(own_out + 3 * __popc(owned & ((1u << e) - 1u)), c);
    }
    if (niso == 1) store3(out, div3(acc, n));
    else {
        Corners cv;
#pragma unroll
        for (int i = 0; i < 8; ++i) cv.v[i] = v[i];
        multi_patch_vertices(tab, cv, g, iso, cfg, lut2, niso, cm, om, out);
    }
}

// Device-side error codes (written with atomicOr to ctx error word).
enum : uint32_t {
    DEV_ERR_TIMEOUT = 1u,
    DEV_ERR_BOUNDS = 2u,
    DEV_ERR_OVERFLOW = 4u,
};

}  // namespace dmc
