// Simple extraction path: per-cell arrays, one look-back scan, per-cell emit.
//
// This path keeps one byte of configuration and one byte of counts per cell
// and a 32-bit vertex and quad offset per cell (10 bytes per cell of scratch).
// It is the straightforward restatement of the reference pipeline
// (dmc.cu:2069-2208) with the reference's compaction replaced by dense
// per-cell offsets; it exists to cross-check the brick path at sizes the CPU
// oracle cannot reach quickly, and as the fallback for shapes the brick path
// does not take.
#include "dmc_device.cuh"
#include "dmc_scan.cuh"
#include "dmc_internal.h"
#include <mutex>

namespace dmc {

constexpr int kSimpleThreads = 256;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;                 // cells per thread in the scan
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ void cell_xyz(uint64_t c, uint3 cells, uint32_t &x, uint32_t &y, uint32_t &z)
{
    uint64_t xy = (uint64_t)cells.x * cells.y;
    z = (uint32_t)(c / xy);
    uint64_t r = c - (uint64_t)z * xy;
    y = (uint32_t)(r / cells.x);
    x = (uint32_t)(r - (uint64_t)y * cells.x);
}

template <class T>
__device__ __forceinline__ void load_corners(const T *vol, uint3 pts, uint32_t x, uint32_t y, uint32_t z, float v[8])
{
    uint64_t sy = pts.x, sz = (uint64_t)pts.x * pts.y;
    uint64_t b = (uint64_t)z * sz + (uint64_t)y * sy + x;
    v[0] = load_sample(vol, b);
    v[1] = load_sample(vol, b + 1);
    v[2] = load_sample(vol, b + sy + 1);
    v[3] = load_sample(vol, b + sy);
    v[4] = load_sample(vol, b + sz);
    v[5] = load_sample(vol, b + sz + 1);
    v[6] = load_sample(vol, b + sz + sy + 1);
    v[7] = load_sample(vol, b + sz + sy);
}

template <class T>
__global__ void __launch_bounds__(kSimpleThreads) simple_classify(const T *vol, uint3 pts, uint3 cells, float iso,
                                                                  uint8_t *cfg, uint64_t n_cells)
{
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t x, y, z;
        cell_xyz(c, cells, x, y, z);
        float v[8];
        load_corners(vol, pts, x, y, z, v);
        cfg[c] = (uint8_t)config_of(v, iso);
    }
}

// Per cell: nv (bits 0-3), owned quads (bits 4-5), lut2 (bit 7); 0 if inactive.
template <class T>
__global__ void __launch_bounds__(kSimpleThreads) simple_count(const T *vol, uint3 pts, uint3 cells, float iso,
                                                               const uint8_t *cfg, uint8_t *cnt, uint64_t n_cells,
                                                               unsigned long long *counters, const DeviceTables *__restrict__ tabp)
{
    const DeviceTables &tab = *tabp;
    uint32_t n_active = 0, n_lut2 = 0, n_dropped = 0;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t cf = cfg[c];
        uint8_t out = 0;
        if (cf != 0 && cf != 0xff) {
            uint32_t x, y, z;
            cell_xyz(c, cells, x, y, z);
            ++n_active;
            bool lut2 = false;
            uint32_t face = tab.amb_face[cf];
            if (face != 0xffu) {
                // face -> neighbour direction (dmc.cu:631-632, 1250-1296)
                int dir = tab.face_dir[face];
                long long nx = x, ny = y, nz = z;
                if (dir == 0) nx++; else if (dir == 1) nx--; else if (dir == 2) ny++;
                else if (dir == 3) ny--; else if (dir == 4) nz++; else nz--;
                if (nx >= 0 && ny >= 0 && nz >= 0 && nx < cells.x && ny < cells.y && nz < cells.z) {
                    uint32_t ncf = cfg[((uint64_t)nz * cells.y + (uint64_t)ny) * cells.x + (uint64_t)nx];
                    lut2 = tab.amb_face[ncf] != 0xffu;
                }
            }
            n_lut2 += lut2;
            float v[8];
            load_corners(vol, pts, x, y, z, v);
            uint32_t info = owned_edge_info(v, iso);
            uint32_t nv = nvert_of(tab, cf, lut2) + __popc(info & 7u);
            uint32_t nq = 0;
#pragma unroll
            for (int s = 0; s < 3; ++s) {
                if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, z, cells)) continue;
                if (owned_sign_change(cf, s)) ++nq; else ++n_dropped;
            }
            out = (uint8_t)(nv | (nq << 4) | (lut2 ? 0x80u : 0u));
        }
        cnt[c] = out;
    }
    // block reduce the counters
    __shared__ uint32_t s_a, s_l, s_d;
    if (threadIdx.x == 0) { s_a = 0; s_l = 0; s_d = 0; }
    __syncthreads();
    if (n_active) atomicAdd(&s_a, n_active);
    if (n_lut2) atomicAdd(&s_l, n_lut2);
    if (n_dropped) atomicAdd(&s_d, n_dropped);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_a) atomicAdd(&counters[0], (unsigned long long)s_a);
        if (s_l) atomicAdd(&counters[1], (unsigned long long)s_l);
        if (s_d) atomicAdd(&counters[2], (unsigned long long)s_d);
    }
}

// Exclusive scan of (nv, nq) over all cells -> per-cell vertex and quad offsets.
__global__ void __launch_bounds__(kScanThreads) simple_scan(const uint8_t *cnt, uint64_t n_cells, ScanCtl ctl,
                                                            uint32_t *vbase, uint32_t *qbase)
{
    __shared__ uint32_t s_slot;
    __shared__ unsigned long long s_warp[kScanThreads / 32 + 1];
    __shared__ unsigned long long s_ex[2];
    const uint32_t tile = claim_tile(ctl.ticket, &s_slot);
    const uint64_t first = (uint64_t)tile * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t nv[kScanItems], nq[kScanItems];
    uint32_t sv = 0, sq = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t c = first + i;
        uint32_t b = c < n_cells ? cnt[c] : 0u;
        nv[i] = b & 15u; nq[i] = (b >> 4) & 3u;
        sv += nv[i]; sq += nq[i];
    }
    unsigned long long tot;
    unsigned long long ex = block_exclusive_scan<kScanThreads>((unsigned long long)sv | ((unsigned long long)sq << 32), s_warp, &tot);
    tile_prefix(ctl, tile, (uint32_t)tot, (uint32_t)(tot >> 32), s_ex);
    unsigned long long bv = s_ex[0] + (uint32_t)ex, bq = s_ex[1] + (uint32_t)(ex >> 32);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        uint64_t c = first + i;
        if (c < n_cells) { vbase[c] = (uint32_t)bv; qbase[c] = (uint32_t)bq; }
        bv += nv[i]; bq += nq[i];
    }
}

template <class T>
__global__ void __launch_bounds__(kSimpleThreads) simple_emit(const T *vol, uint3 pts, uint3 cells, float iso, float3 mn, float3 rng,
                                                              const uint8_t *cfg, const uint8_t *cnt,
                                                              const uint32_t *vbase, const uint32_t *qbase, uint64_t n_cells,
                                                              float *verts, uint64_t vcap, uint32_t *quads, uint64_t qcap,
                                                              uint32_t *tris, uint32_t *err, const DeviceTables *__restrict__ tabp)
{
    const DeviceTables &tab = *tabp;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t b = cnt[c];
        if (b == 0) continue;
        uint32_t cf = cfg[c];
        bool lut2 = (b & 0x80u) != 0;
        uint32_t nv = b & 15u, nq = (b >> 4) & 3u;
        uint32_t x, y, z;
        cell_xyz(c, cells, x, y, z);
        float v[8];
        load_corners(vol, pts, x, y, z, v);
        uint32_t info = owned_edge_info(v, iso);
        uint32_t niso = nvert_of(tab, cf, lut2);
        uint64_t vb = vbase[c];
        if (vb + nv > vcap) { atomicOr(err, DEV_ERR_OVERFLOW); continue; }
        Geo g = cell_geo(x, y, z, cells, rng, mn);
        dual_vertices(tab, v, g, iso, cf, lut2, x, y, z, niso, verts + 3 * vb);
        owned_edge_vertices(v, g, iso, info, verts + 3 * (vb + niso));
        if (!nq) continue;
        uint64_t q = qbase[c];
        if (q + nq > qcap) { atomicOr(err, DEV_ERR_OVERFLOW); continue; }
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, z, cells) || !owned_sign_change(cf, s)) continue;
            bool ccw = (info >> (s + 3)) & 1u;
            uint32_t idx[4];
#pragma unroll
            for (int it = 0; it < 4; ++it) {
                int k = ccw ? it : (4 - it) & 3;
                int re, dx, dy, dz;
                ring_entry(s, k, re, dx, dy, dz);
                uint64_t rc = ((uint64_t)(z + dz) * cells.y + (y + dy)) * cells.x + (x + dx);
                uint32_t rb = cnt[rc];
                uint32_t m = lut_m(tab, cfg[rc], (rb & 0x80u) != 0, re);
                if (m == 0xffu) { atomicOr(err, DEV_ERR_BOUNDS); m = 0; }
                idx[it] = vbase[rc] + m;
            }
            uint4 qv = make_uint4(idx[0], idx[1], idx[2], idx[3]);
            reinterpret_cast<uint4 *>(quads)[q] = qv;
            if (tris) {
                uint32_t *t = tris + 6 * q;
                t[0] = idx[0]; t[1] = idx[1]; t[2] = idx[2];
                t[3] = idx[2]; t[4] = idx[3]; t[5] = idx[0];
            }
            ++q;
        }
    }
}

// ---------------------------------------------------------------------------
// Vertex smoothing (dmc.cu:1710-1981, driven at 2157-2169).  One iteration:
// simple_smooth_edges moves the crossing of every owned edge that has a quad
// onto the split triangle of its ring of four dual vertices, projected along
// the edge's axis; simple_smooth_duals then recomputes every dual vertex as
// the mean of its patch's crossings.  Single precision with explicit rounding
// (no fused multiply-add), correctly rounded square root and division, in the
// reference's operand order.  Two restatements of the reference's arithmetic:
// lengths are normalised with 1/sqrt instead of the approximate rsqrtf, and a
// convex quadrilateral is split at the corner with the smallest cosine
// instead of the largest acosf angle (the same corner except where acosf
// rounds two cosines to one angle).

__device__ __forceinline__ bool cross_z_positive(float lx, float ly, float mx, float my, float rx, float ry)
{
    const float dx1 = __fsub_rn(rx, mx), dy1 = __fsub_rn(ry, my);
    const float dx2 = __fsub_rn(lx, mx), dy2 = __fsub_rn(ly, my);
    return __fsub_rn(__fmul_rn(dx1, dy2), __fmul_rn(dx2, dy1)) >= 0.f;
}

__device__ __forceinline__ float corner_cos(float lx, float ly, float mx, float my, float rx, float ry)
{
    float ux = __fsub_rn(lx, mx), uy = __fsub_rn(ly, my), vx = __fsub_rn(rx, mx), vy = __fsub_rn(ry, my);
    const float iu = __fdiv_rn(1.f, __fsqrt_rn(__fadd_rn(__fmul_rn(ux, ux), __fmul_rn(uy, uy))));
    const float iv = __fdiv_rn(1.f, __fsqrt_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy))));
    ux = __fmul_rn(ux, iu); uy = __fmul_rn(uy, iu); vx = __fmul_rn(vx, iv); vy = __fmul_rn(vy, iv);
    return __fadd_rn(__fmul_rn(ux, vx), __fmul_rn(uy, vy));
}

// is_inside_triangle (dmc.cu:1894-1912) in the projection plane
__device__ __forceinline__ bool inside_triangle(const float p0[2], const float p1[2], const float p2[2], float ox,
                                                float oy, float &alpha, float &beta, float &gamma)
{
    const float v0x = __fsub_rn(p1[0], p0[0]), v0y = __fsub_rn(p1[1], p0[1]);
    const float v1x = __fsub_rn(p2[0], p0[0]), v1y = __fsub_rn(p2[1], p0[1]);
    const float v2x = __fsub_rn(ox, p0[0]), v2y = __fsub_rn(oy, p0[1]);
    const float d00 = __fadd_rn(__fmul_rn(v0x, v0x), __fmul_rn(v0y, v0y));
    const float d10 = __fadd_rn(__fmul_rn(v1x, v0x), __fmul_rn(v1y, v0y));
    const float d11 = __fadd_rn(__fmul_rn(v1x, v1x), __fmul_rn(v1y, v1y));
    const float d20 = __fadd_rn(__fmul_rn(v2x, v0x), __fmul_rn(v2y, v0y));
    const float d21 = __fadd_rn(__fmul_rn(v2x, v1x), __fmul_rn(v2y, v1y));
    const float inv = __fdiv_rn(1.f, __fsub_rn(__fmul_rn(d00, d11), __fmul_rn(d10, d10)));
    beta = __fmul_rn(__fsub_rn(__fmul_rn(d11, d20), __fmul_rn(d10, d21)), inv);
    gamma = __fmul_rn(__fsub_rn(__fmul_rn(d00, d21), __fmul_rn(d10, d20)), inv);
    alpha = __fsub_rn(__fsub_rn(1.f, beta), gamma);
    return (-1e-4 < (double)beta) && (-1e-4 < (double)gamma) && ((double)__fadd_rn(beta, gamma) < 1.0 + 1e-4);
}

// New crossing of owned edge s (0: edge 6, 1: 9, 2: 10) from its quad ring;
// false when it stays (complex quadrilateral, or the edge outside both halves).
__device__ bool smooth_edge(const float *__restrict__ verts, const uint32_t ring[4], int s, float ox, float oy,
                            float out[3])
{
    const int ax = s == 2 ? 1 : 0, ay = s == 0 ? 1 : 2;     // 6: xy, 9: xz, 10: yz
    float P[4][2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        P[i][0] = verts[3 * (uint64_t)ring[i] + ax];
        P[i][1] = verts[3 * (uint64_t)ring[i] + ay];
    }
    int npos = 0, ipos = 0, ineg = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int l = (i + 3) & 3, r = (i + 1) & 3;
        if (cross_z_positive(P[l][0], P[l][1], P[i][0], P[i][1], P[r][0], P[r][1])) { ++npos; ipos = i; }
        else ineg = i;
    }
    if (npos == 2) return false;
    int split0;
    if (npos == 0 || npos == 4) {
        float best = corner_cos(P[3][0], P[3][1], P[0][0], P[0][1], P[1][0], P[1][1]);
        split0 = 0;
#pragma unroll
        for (int i = 1; i < 4; ++i) {
            const int l = (i + 3) & 3, r = (i + 1) & 3;
            const float c = corner_cos(P[l][0], P[l][1], P[i][0], P[i][1], P[r][0], P[r][1]);
            if (c < best) { best = c; split0 = i; }
        }
    } else {
        split0 = npos == 1 ? ipos : ineg;
    }
    const int split1 = (split0 + 2) & 3;
    float al, be, ga;
    int a, b, c;
    if (inside_triangle(P[split0], P[(split0 + 1) & 3], P[split1], ox, oy, al, be, ga)) {
        a = split0; b = (split0 + 1) & 3; c = split1;
    } else if (inside_triangle(P[split1], P[(split1 + 1) & 3], P[split0], ox, oy, al, be, ga)) {
        a = split1; b = (split1 + 1) & 3; c = split0;
    } else {
        return false;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float t = __fmul_rn(al, verts[3 * (uint64_t)ring[a] + k]);
        t = __fadd_rn(t, __fmul_rn(be, verts[3 * (uint64_t)ring[b] + k]));
        t = __fadd_rn(t, __fmul_rn(ga, verts[3 * (uint64_t)ring[c] + k]));
        out[k] = t;
    }
    return true;
}

// bipolar/ccw bits of each active cell's own edges, for the smoothing passes
template <class T>
__global__ void __launch_bounds__(kSimpleThreads) simple_info(const T *vol, uint3 pts, uint3 cells, float iso,
                                                              const uint8_t *cnt, uint8_t *inf, uint64_t n_cells)
{
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        if (!cnt[c]) continue;
        uint32_t x, y, z;
        cell_xyz(c, cells, x, y, z);
        float v[8];
        load_corners(vol, pts, x, y, z, v);
        inf[c] = (uint8_t)owned_edge_info(v, iso);
    }
}

__global__ void __launch_bounds__(kSimpleThreads) simple_smooth_edges(uint3 cells, float3 mn, float3 rng,
        const uint8_t *cfg, const uint8_t *cnt, const uint8_t *inf, const uint32_t *vbase, const uint32_t *qbase,
        uint64_t n_cells, float *verts, const uint32_t *quads, const DeviceTables *__restrict__ tabp)
{
    const DeviceTables &tab = *tabp;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = cnt[c];
        if (!((b >> 4) & 3u)) continue;
        uint32_t x, y, z;
        cell_xyz(c, cells, x, y, z);
        const uint32_t cf = cfg[c], info = inf[c];
        const uint32_t niso = nvert_of(tab, cf, (b & 0x80u) != 0);
        const float x1 = ijk_to_xyz(x + 1, cells.x, rng.x, mn.x);
        const float y1 = ijk_to_xyz(y + 1, cells.y, rng.y, mn.y);
        const float z1 = ijk_to_xyz(z + 1, cells.z, rng.z, mn.z);
        uint64_t q = qbase[c];
        for (int s = 0; s < 3; ++s) {
            if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, z, cells) || !owned_sign_change(cf, s)) continue;
            const uint4 r4 = reinterpret_cast<const uint4 *>(quads)[q++];
            const uint32_t ring[4] = {r4.x, r4.y, r4.z, r4.w};
            float nv[3];
            if (smooth_edge(verts, ring, s, s == 2 ? y1 : x1, s == 0 ? y1 : z1, nv)) {
                const uint64_t ev = (uint64_t)vbase[c] + niso + __popc(info & ((1u << s) - 1u));
                verts[3 * ev + 0] = nv[0]; verts[3 * ev + 1] = nv[1]; verts[3 * ev + 2] = nv[2];
            }
        }
    }
}

// owner-edge slot (0: edge 6, 1: 9, 2: 10) of each cell edge, 2 bits per edge
constexpr uint32_t kOwnerSlot = 0x660066u;   // edges 0..11: 2,1,2,1,0,0,0,0,2,1,2,1

__global__ void __launch_bounds__(kSimpleThreads) simple_smooth_duals(uint3 cells, const uint8_t *cfg,
        const uint8_t *cnt, const uint8_t *inf, const uint32_t *vbase, uint64_t n_cells, float *verts,
        const DeviceTables *__restrict__ tabp)
{
    const DeviceTables &tab = *tabp;
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells; c += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b = cnt[c];
        if (!b) continue;
        uint32_t x, y, z;
        cell_xyz(c, cells, x, y, z);
        const uint32_t cf = cfg[c];
        const bool l2 = (b & 0x80u) != 0;
        const uint32_t niso = nvert_of(tab, cf, l2);
        float3 acc[4];
        uint32_t n4[4] = {0, 0, 0, 0};
        acc[0] = acc[1] = acc[2] = acc[3] = make_float3(0.f, 0.f, 0.f);
#pragma unroll 1
        for (int e = 0; e < 12; ++e) {
            const uint32_t m = lut_m(tab, cf, l2, e);
            if (m == 0xffu) continue;
            if ((owner_dx(e) < 0 && x == 0) || (owner_dy(e) < 0 && y == 0) || (owner_dz(e) < 0 && z == 0)) continue;
            const uint64_t o = ((uint64_t)(z + owner_dz(e)) * cells.y + (y + owner_dy(e))) * cells.x + (x + owner_dx(e));
            const uint32_t slot = (kOwnerSlot >> (2 * e)) & 3u;
            const uint64_t ev = (uint64_t)vbase[o] + nvert_of(tab, cfg[o], (cnt[o] & 0x80u) != 0) +
                                __popc(inf[o] & ((1u << slot) - 1u));
            const float3 src = make_float3(verts[3 * ev], verts[3 * ev + 1], verts[3 * ev + 2]);
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (m == (uint32_t)k) { acc[k] = n4[k] ? add3(acc[k], src) : src; n4[k]++; }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if ((uint32_t)k < niso && n4[k]) store3(verts + 3 * ((uint64_t)vbase[c] + k), div3(acc[k], n4[k]));
    }
}

// ---------------------------------------------------------------------------
// host side

static int grid_for(uint64_t n, int threads, int num_sms)
{
    uint64_t blocks = (n + threads - 1) / threads;
    uint64_t cap = (uint64_t)num_sms * 16;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

template <class T>
static dmc_status simple_run_t(Ctx *ctx, const T *vol, const ExtractArgs &a, cudaStream_t st)
{
    const uint64_t C = a.n_cells;
    const uint64_t n_tiles64 = (C + kScanTile - 1) / kScanTile;
    if (n_tiles64 >= (1ull << 31)) return DMC_ERR_UNSUPPORTED;
    const uint32_t n_tiles = (uint32_t)n_tiles64;
    // scratch: cfg C, cnt C, vbase 4C, qbase 4C, tiles
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    size_t o_cfg = carve(C), o_cnt = carve(C), o_vb = carve(4 * C), o_qb = carve(4 * C);
    size_t o_tiles = carve(sizeof(TileState) * n_tiles);
    const size_t o_inf = a.num_smooth ? carve(C) : 0;
    dmc_status s = ctx_reserve_scratch(ctx, off);
    if (s != DMC_OK) return s;
    uint8_t *base = (uint8_t *)ctx->scratch;
    uint8_t *cfg = base + o_cfg, *cnt = base + o_cnt;
    uint32_t *vb = (uint32_t *)(base + o_vb), *qb = (uint32_t *)(base + o_qb);
    TileState *tiles = (TileState *)(base + o_tiles);

    CUDA_TRY(cudaMemsetAsync(tiles, 0, sizeof(TileState) * n_tiles, st));
    CUDA_TRY(cudaMemsetAsync(ctx->d_ctl, 0, sizeof(DevCtl), st));
    const int g = grid_for(C, kSimpleThreads, ctx->num_sms);
    simple_classify<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, cfg, C);
    simple_count<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, cfg, cnt, C, ctx->d_ctl->counters, ctx->d_tab);
    ScanCtl ctl;
    ctl.tiles = tiles; ctl.ticket = &ctx->d_ctl->ticket; ctl.err = &ctx->d_ctl->err;
    ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = n_tiles;
    simple_scan<<<n_tiles, kScanThreads, 0, st>>>(cnt, C, ctl, vb, qb);
    CUDA_TRY(cudaGetLastError());
    // totals decide whether the caller's buffers are large enough
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (ctx->h_ctl->err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    const uint64_t V = ctx->h_ctl->totals[0], Q = ctx->h_ctl->totals[1];
    *a.n_vertices = V; *a.n_quads = Q;
    ctx->stats.n_active_cells = ctx->h_ctl->counters[0];
    ctx->stats.n_lut2_cells = ctx->h_ctl->counters[1];
    ctx->stats.n_dropped_quads = ctx->h_ctl->counters[2];
    if (V >= 0xFFFFFFFFull || Q >= 0xFFFFFFFFull) return DMC_ERR_OUTPUT_OVERFLOW;
    if (a.sizing_only) return DMC_OK;
    if (V > a.vcap || Q > a.qcap) return DMC_ERR_OUTPUT_OVERFLOW;
    simple_emit<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, a.mn, a.rng, cfg, cnt, vb, qb, C,
                                                  a.verts, a.vcap, a.quads, a.qcap, a.tris, &ctx->d_ctl->err, ctx->d_tab);
    CUDA_TRY(cudaGetLastError());
    if (a.num_smooth) {
        uint8_t *inf = base + o_inf;
        simple_info<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, cnt, inf, C);
        for (uint32_t it = 0; it < a.num_smooth; ++it) {
            simple_smooth_edges<<<g, kSimpleThreads, 0, st>>>(a.cells, a.mn, a.rng, cfg, cnt, inf, vb, qb, C, a.verts,
                                                               a.quads, ctx->d_tab);
            simple_smooth_duals<<<g, kSimpleThreads, 0, st>>>(a.cells, cfg, cnt, inf, vb, C, a.verts, ctx->d_tab);
        }
        CUDA_TRY(cudaGetLastError());
    }
    return DMC_OK;
}

dmc_status simple_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st)
{
    if (a.dtype == DMC_F32) return simple_run_t<float>(ctx, (const float *)a.vol, a, st);
    return simple_run_t<uint16_t>(ctx, (const uint16_t *)a.vol, a, st);
}

// ---------------------------------------------------------------------------
// No-allocation variant of the simple path (dmc_extract_device_noalloc).
//
// For callers that must not have a library allocate device memory on their
// behalf: processes whose device memory is held by a pool allocator that has
// reserved what is free (a framework's caching allocator, an application heap),
// so that a cudaMalloc from here would fail or fragment it; and latency-bound
// loops sharing the GPU with other streams, where cudaMalloc / cudaFree may
// synchronise the device and stall them.  Everything the pipeline needs --
// lookup tables, control block, per-cell arrays and scan tile states -- lives
// in one fixed array in the module's global memory, sized for at most
// kNoAllocMaxCells cells.  Every call takes its address with
// cudaGetSymbolAddress (host code must not pass the array's name itself to a
// kernel); the first call on a device, and the first after its context was
// replaced, also uploads the tables and synchronises the device, so make that
// first call before any stream capture.  Per call, only the control
// block and the scan tile states must start at zero (cleared with
// cudaMemsetAsync on the caller's stream); the per-cell arrays are fully
// rewritten.  There is one array per device, so calls on the same device must
// not overlap in time: concurrent calls from several host threads race on it.

constexpr uint64_t kNoAllocMaxCells = DMC_NOALLOC_MAX_CELLS;
constexpr size_t na_align(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr uint64_t kNoAllocTiles = (kNoAllocMaxCells + kScanTile - 1) / kScanTile;
constexpr size_t kNaTab = 0;
constexpr size_t kNaCtl = kNaTab + na_align(sizeof(DeviceTables));
constexpr size_t kNaCfg = kNaCtl + na_align(sizeof(DevCtl));
constexpr size_t kNaCnt = kNaCfg + na_align(kNoAllocMaxCells);
constexpr size_t kNaVb = kNaCnt + na_align(kNoAllocMaxCells);
constexpr size_t kNaQb = kNaVb + na_align(4 * kNoAllocMaxCells);
constexpr size_t kNaTiles = kNaQb + na_align(4 * kNoAllocMaxCells);
constexpr size_t kNoAllocBytes = kNaTiles + na_align(sizeof(TileState) * kNoAllocTiles);   // ~10.1 MiB

static __device__ __align__(256) uint8_t g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_noalloc_setup_mu;
static uint8_t *g_noalloc_base[256];          // per device, set by the set-up
static unsigned long long g_noalloc_ctx[256]; // id of the CUDA context that set-up ran in (0: none yet)

// Unique id of the calling thread's current CUDA context (cuCtxGetId, which
// never repeats within a process), taken through the runtime's driver entry
// points so the library needs no link against libcuda.  0 when unavailable.
static unsigned long long current_context_id()
{
    typedef int (*GetCurrent)(void **);
    typedef int (*GetId)(void *, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)f;
    });
    void *c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != 0 || !c || get_id(c, &id) != 0) return 0;
    return id;
}

// Set-up, once per device and CUDA context: the array's device address
// (cudaGetSymbolAddress with the device current) and the lookup tables.  The
// upload is followed by a device synchronisation, so the tables are complete
// before any kernel on any stream (including non-blocking ones) reads them.
// A context that replaced an earlier one on the device (after
// cudaDeviceReset) gets a fresh set-up: its array is a new allocation.
static dmc_status noalloc_setup(int device, uint8_t **base)
{
    if (device < 0 || device >= 256) return DMC_ERR_INVALID_ARG;
    // Looked up on every call: it also makes the device's primary context
    // current, which the context id below needs.
    void *p = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(g_noalloc_setup_mu);
    if (g_noalloc_base[device] != (uint8_t *)p || ctx == 0 || ctx != g_noalloc_ctx[device]) {
        DeviceTables h;
        fill_tables(h);
        CUDA_TRY(cudaMemcpy((uint8_t *)p + kNaTab, &h, sizeof(DeviceTables), cudaMemcpyHostToDevice));
        CUDA_TRY(cudaDeviceSynchronize());
        g_noalloc_base[device] = (uint8_t *)p;
        g_noalloc_ctx[device] = ctx;
    }
    *base = g_noalloc_base[device];
    return DMC_OK;
}

template <class T>
static dmc_status noalloc_run_t(uint8_t *base, const T *vol, const ExtractArgs &a, int num_sms, cudaStream_t st)
{
    const uint64_t C = a.n_cells;
    const uint32_t n_tiles = (uint32_t)((C + kScanTile - 1) / kScanTile);
    const DeviceTables *tab = (const DeviceTables *)(base + kNaTab);
    DevCtl *ctl_d = (DevCtl *)(base + kNaCtl);
    uint8_t *cfg = base + kNaCfg, *cnt = base + kNaCnt;
    uint32_t *vb = (uint32_t *)(base + kNaVb), *qb = (uint32_t *)(base + kNaQb);
    TileState *tiles = (TileState *)(base + kNaTiles);
    CUDA_TRY(cudaMemsetAsync(tiles, 0, sizeof(TileState) * n_tiles, st));
    CUDA_TRY(cudaMemsetAsync(ctl_d, 0, sizeof(DevCtl), st));
    const int g = grid_for(C, kSimpleThreads, num_sms);
    simple_classify<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, cfg, C);
    simple_count<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, cfg, cnt, C, ctl_d->counters, tab);
    ScanCtl ctl;
    ctl.tiles = tiles; ctl.ticket = &ctl_d->ticket; ctl.err = &ctl_d->err;
    ctl.totals = ctl_d->totals; ctl.n_tiles = n_tiles;
    simple_scan<<<n_tiles, kScanThreads, 0, st>>>(cnt, C, ctl, vb, qb);
    CUDA_TRY(cudaGetLastError());
    DevCtl h;   // pageable host copy: no pinned buffer to allocate
    CUDA_TRY(cudaMemcpyAsync(&h, ctl_d, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (h.err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    *a.n_vertices = h.totals[0]; *a.n_quads = h.totals[1];
    if (a.sizing_only) return DMC_OK;
    if (h.totals[0] > a.vcap || h.totals[1] > a.qcap) return DMC_ERR_OUTPUT_OVERFLOW;
    simple_emit<T><<<g, kSimpleThreads, 0, st>>>(vol, a.pts, a.cells, a.iso, a.mn, a.rng, cfg, cnt, vb, qb, C,
                                                  a.verts, a.vcap, a.quads, a.qcap, a.tris, &ctl_d->err, tab);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(&h, ctl_d, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (h.err & DEV_ERR_OVERFLOW) return DMC_ERR_OUTPUT_OVERFLOW;
    if (h.err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    return DMC_OK;
}

}  // namespace dmc

extern "C" dmc_status dmc_extract_device_noalloc(const dmc_volume *vol, const float xyz_min[3],
                                                 const float xyz_max[3], float iso, float *d_vertices,
                                                 uint64_t vertex_capacity, uint32_t *d_quads, uint64_t quad_capacity,
                                                 uint32_t *d_triangles, uint64_t *n_vertices, uint64_t *n_quads,
                                                 void *stream)
{
    dmc::NvtxRange nvtx("dmc_extract_device_noalloc");
    using namespace dmc;
    if (!vol || !vol->data || !xyz_min || !xyz_max || !n_vertices || !n_quads) return DMC_ERR_INVALID_ARG;
    if (vol->dtype != DMC_F32 && vol->dtype != DMC_U16) return DMC_ERR_INVALID_ARG;
    if ((vertex_capacity && !d_vertices) || (quad_capacity && !d_quads)) return DMC_ERR_INVALID_ARG;
    *n_vertices = 0; *n_quads = 0;
    ExtractArgs a{};
    a.vol = vol->data;
    a.dtype = vol->dtype;
    a.pts = make_uint3(vol->dims[0], vol->dims[1], vol->dims[2]);
    a.cells = make_uint3(vol->dims[0] ? vol->dims[0] - 1 : 0, vol->dims[1] ? vol->dims[1] - 1 : 0,
                         vol->dims[2] ? vol->dims[2] - 1 : 0);
    if (!cell_count(a.cells, &a.n_cells) || a.n_cells > kNoAllocMaxCells) return DMC_ERR_TOO_LARGE;
    a.iso = iso;
    a.mn = make_float3(xyz_min[0], xyz_min[1], xyz_min[2]);
    a.rng = make_float3(xyz_max[0] - xyz_min[0], xyz_max[1] - xyz_min[1], xyz_max[2] - xyz_min[2]);
    a.verts = d_vertices; a.vcap = vertex_capacity;
    a.quads = d_quads; a.qcap = quad_capacity;
    a.tris = d_triangles;
    a.n_vertices = n_vertices; a.n_quads = n_quads;
    a.sizing_only = !d_vertices && !d_quads && !d_triangles;
    int device = 0, num_sms = 0;
    CUDA_TRY(cudaGetDevice(&device));
    CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device));
    uint8_t *base = nullptr;
    dmc_status s = noalloc_setup(device, &base);
    if (s != DMC_OK) return s;
    if (a.n_cells == 0) return DMC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (a.dtype == DMC_F32) return noalloc_run_t<float>(base, (const float *)a.vol, a, num_sms, st);
    return noalloc_run_t<uint16_t>(base, (const uint16_t *)a.vol, a, num_sms, st);
}

