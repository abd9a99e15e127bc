// Brick path: bit-sliced classification over z-sweeping bricks, a segment
// scan with decoupled look-back, and an emit sweep that writes vertices and
// quads at their final positions.
//
// Layout.  A brick covers W = 32*NW cell columns (one thread per column) and
// 32 cell rows and sweeps a run of z planes.  For each point plane, every
// thread loads its column's 34 samples (rows y0..y0+33, coalesced along x)
// and keeps only one bit per sample, "below the isovalue", packed in a 64-bit
// mask.  A cell's configuration is then a handful of shifts on the masks of
// two neighbouring columns in two planes; activity for all 33 rows of a
// column is ~12 bitwise operations.  Only active cells (a few percent) take
// the per-cell path (2B/3B test, counts, positions).
//
// Ordering.  Output order is the reference's: ascending cell index (x fastest,
// utils.hpp:72), so a brick's cells at one plane and row form a contiguous
// output range, a "segment" (plane k, row j, x segment xs).  The count sweep
// writes per-segment (vertices, quads); a decoupled look-back scan turns them
// into offsets; the emit sweep recomputes the classification, ranks the
// active cells inside each segment and writes positions and quads.
//
// Halo.  Quads of a cell reference the dual vertices of its +x, +y, +z
// neighbours (dmc.cu:1636-1664).  The emit sweep therefore also classifies
// the first cell column of the next x segment (its vertices start exactly at
// that segment's offset) and the first row of the next brick (ranked within
// its own segment), and defers the quads of plane k until plane k+1 is known.
#include "dmc_device.cuh"
#include "dmc_scan.cuh"
#include "dmc_internal.h"

namespace dmc {

namespace brick {

constexpr int NW = 4;                 // warps per brick
constexpr int W = 32 * NW;            // own cell columns
constexpr int NT = 32 * NW;           // threads
constexpr int ROWS = 32;              // own cell rows
constexpr int HROWS = ROWS + 1;       // with the halo row
constexpr int HCOLS = W + 1;          // with the halo column
constexpr int MAXL = HROWS * HCOLS;   // list capacity (every cell active)
constexpr int ZC = 32;                // planes per brick in the two-pass form
constexpr int SCAN_NT = 256, SCAN_ITEMS = 8, SCAN_TILE = SCAN_NT * SCAN_ITEMS;

struct Geom {
    uint3 pts, cells;
    uint32_t nxs, nyb, nzc, zc;
    float iso;
    float3 mn, rng;
};

__device__ __forceinline__ uint64_t seg_index(const Geom &g, uint32_t k, uint32_t j, uint32_t xs)
{
    return ((uint64_t)k * g.cells.y + j) * g.nxs + xs;
}

template <class T>
__device__ __forceinline__ float sample_at(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z)
{
    return load_sample(vol, ((uint64_t)z * g.pts.y + y) * g.pts.x + x);
}

// Masks of point plane p for columns x0 .. x0+W+1 into s_mask[0..W+2).
// Bit r of column c: sample (x0+c, y0+r, p) < iso, r in 0..33.  Samples
// outside the volume read as 0 (their cells are never active).
template <class T>
__device__ __forceinline__ void load_masks(const T *vol, const Geom &g, uint32_t x0, uint32_t y0, uint32_t p,
                                           uint64_t *s_mask)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const bool pz = p < g.pts.z;
    {
        const uint32_t x = x0 + t;
        uint32_t lo = 0, hi = 0;
        if (pz && x < g.pts.x) {
            const T *col = vol + (uint64_t)p * g.pts.y * g.pts.x + x;
            const uint32_t nrow = g.pts.y > y0 ? min(34u, g.pts.y - y0) : 0u;
            const uint64_t sx = g.pts.x;
            if (nrow == 34) {
                float v[34];
#pragma unroll
                for (int r = 0; r < 34; ++r) v[r] = load_sample(col, (uint64_t)(y0 + r) * sx);
#pragma unroll
                for (int r = 0; r < 32; ++r) lo |= (v[r] < g.iso ? 1u : 0u) << r;
                hi = (v[32] < g.iso ? 1u : 0u) | (v[33] < g.iso ? 2u : 0u);
            } else {
                for (uint32_t r = 0; r < nrow; ++r) {
                    float v = load_sample(col, (uint64_t)(y0 + r) * sx);
                    if (v < g.iso) { if (r < 32) lo |= 1u << r; else hi |= 1u << (r - 32); }
                }
            }
        }
        s_mask[t] = (uint64_t)lo | ((uint64_t)hi << 32);
    }
    if (warp == NW - 1) {
#pragma unroll
        for (int hc = 0; hc < 2; ++hc) {
            const uint32_t x = x0 + W + hc;
            const bool okx = pz && x < g.pts.x;
            const uint32_t y = y0 + lane, y2 = y0 + 32 + lane;
            bool b = okx && y < g.pts.y && sample_at(vol, g, x, y, p) < g.iso;
            bool b2 = okx && lane < 2 && y2 < g.pts.y && sample_at(vol, g, x, y2, p) < g.iso;
            uint32_t lo = __ballot_sync(0xffffffffu, b);
            uint32_t hi = __ballot_sync(0xffffffffu, b2) & 3u;
            if (lane == 0) s_mask[W + hc] = (uint64_t)lo | ((uint64_t)hi << 32);
        }
    }
}

// Rows r (bit r) whose cell (column with masks A,B bottom and C,D top, A/C at
// x, B/D at x+1) has corners on both sides of the isovalue.
__device__ __forceinline__ uint64_t active_rows(uint64_t A, uint64_t B, uint64_t C, uint64_t D)
{
    uint64_t a = A & B & C & D, o = A | B | C | D;
    return (o | (o >> 1)) & ~(a & (a >> 1));
}

// Configuration of the cell in row r from the four column masks
// (corner order of dmc.cu:1044-1054).
__device__ __forceinline__ uint32_t cfg_from_masks(uint64_t A, uint64_t B, uint64_t C, uint64_t D, int r)
{
    uint32_t a = (uint32_t)(A >> r), b = (uint32_t)(B >> r), c = (uint32_t)(C >> r), d = (uint32_t)(D >> r);
    return (a & 1u) | ((b & 1u) << 1) | ((b & 2u) << 1) | ((a & 2u) << 2) |
           ((c & 1u) << 4) | ((d & 1u) << 5) | ((d & 2u) << 5) | ((c & 2u) << 6);
}

template <class T>
__device__ __forceinline__ uint32_t cfg_global(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z)
{
    float v[8];
    v[0] = sample_at(vol, g, x, y, z);         v[1] = sample_at(vol, g, x + 1, y, z);
    v[2] = sample_at(vol, g, x + 1, y + 1, z); v[3] = sample_at(vol, g, x, y + 1, z);
    v[4] = sample_at(vol, g, x, y, z + 1);     v[5] = sample_at(vol, g, x + 1, y, z + 1);
    v[6] = sample_at(vol, g, x + 1, y + 1, z + 1); v[7] = sample_at(vol, g, x, y + 1, z + 1);
    return config_of(v, g.iso);
}

// 2B/3B correction (dmc.cu:1232-1371): the cell uses LUT2 when its config is
// one of the 36 ambiguous ones and the face neighbour's config is too.  The
// neighbour's config comes from the masks when it lies in the window
// (columns 0..W, rows 0..32 of plane k), otherwise from eight global loads.
template <class T>
__device__ __forceinline__ bool needs_lut2(const T *vol, const Geom &g, const DeviceTables &tab, uint32_t cfg,
                                           const uint64_t *mk, const uint64_t *mk1, int c, int r,
                                           uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t face = tab.amb_face[cfg];
    if (face == 0xffu) return false;
    int dir = tab.face_dir[face];
    int dx = dir == 0 ? 1 : (dir == 1 ? -1 : 0);
    int dy = dir == 2 ? 1 : (dir == 3 ? -1 : 0);
    int dz = dir == 4 ? 1 : (dir == 5 ? -1 : 0);
    long long nx = (long long)x + dx, ny = (long long)y + dy, nz = (long long)z + dz;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= g.cells.x || ny >= g.cells.y || nz >= g.cells.z) return false;
    uint32_t ncfg;
    int nc = c + dx, nr = r + dy;
    if (dz == 0 && nc >= 0 && nc <= W && nr >= 0 && nr <= ROWS)
        ncfg = cfg_from_masks(mk[nc], mk[nc + 1], mk1[nc], mk1[nc + 1], nr);
    else
        ncfg = cfg_global(vol, g, (uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
    return tab.amb_face[ncfg] != 0xffu;
}

// Reference bipolarity and ccw bits of the cell's own edges, from corners
// 2, 5, 6, 7 (dmc.cu:1199-1216); see owned_edge_info.
template <class T>
__device__ __forceinline__ uint32_t owned_info_global(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z)
{
    float v2 = sample_at(vol, g, x + 1, y + 1, z), v5 = sample_at(vol, g, x + 1, y, z + 1);
    float v6 = sample_at(vol, g, x + 1, y + 1, z + 1), v7 = sample_at(vol, g, x, y + 1, z + 1);
    uint32_t info = 0;
    if (ref_bipolar(v2, v6, g.iso)) info |= 1u | (v2 <= g.iso ? 8u : 0u);
    if (ref_bipolar(v5, v6, g.iso)) info |= 2u | (v5 <= g.iso ? 16u : 0u);
    if (ref_bipolar(v7, v6, g.iso)) info |= 4u | (v7 <= g.iso ? 32u : 0u);
    return info;
}

__device__ __forceinline__ uint32_t quad_count(uint32_t info, uint32_t cfg, uint32_t x, uint32_t y, uint32_t z,
                                               uint3 cells, uint32_t *dropped)
{
    uint32_t nq = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, z, cells)) continue;
        if (owned_sign_change(cfg, s)) ++nq; else ++*dropped;
    }
    return nq;
}

__device__ __forceinline__ uint64_t row_valid_mask(uint32_t y0, uint32_t cy, int rows)
{
    uint32_t n = cy > y0 ? min((uint32_t)rows, cy - y0) : 0u;
    return n >= 64 ? ~0ull : ((1ull << n) - 1ull);
}

// ---------------------------------------------------------------------------
// count sweep: per-segment (vertices, quads)

template <class T>
__global__ void __launch_bounds__(NT) brick_count(const T *__restrict__ vol, Geom g, const DeviceTables *__restrict__ tabp,
                                                  uint2 *__restrict__ seg_cnt, unsigned long long *counters)
{
    __shared__ uint64_t s_mask[2][W + 2];
    __shared__ uint32_t s_rv[ROWS], s_rq[ROWS];
    __shared__ uint32_t s_stat[3];
    const DeviceTables &tab = *tabp;
    const int t = threadIdx.x;
    const uint32_t xs = blockIdx.x, yb = blockIdx.y, zb = blockIdx.z;
    const uint32_t x0 = xs * W, y0 = yb * ROWS, z0 = zb * g.zc;
    const uint32_t z1 = min(z0 + g.zc, g.cells.z);
    const uint32_t x = x0 + t;
    const bool colok = x < g.cells.x;
    const uint64_t rowmask = row_valid_mask(y0, g.cells.y, ROWS);
    uint32_t n_act = 0, n_l2 = 0, n_drop = 0;
    if (t < 3) s_stat[t] = 0;

    load_masks(vol, g, x0, y0, z0, s_mask[z0 & 1]);
    for (uint32_t k = z0; k < z1; ++k) {
        if (t < ROWS) { s_rv[t] = 0; s_rq[t] = 0; }
        load_masks(vol, g, x0, y0, k + 1, s_mask[(k + 1) & 1]);
        __syncthreads();
        const uint64_t *mk = s_mask[k & 1], *mk1 = s_mask[(k + 1) & 1];
        uint64_t act = colok ? active_rows(mk[t], mk[t + 1], mk1[t], mk1[t + 1]) & rowmask : 0ull;
        while (act) {
            const int r = __ffsll((long long)act) - 1;
            act &= act - 1;
            const uint32_t y = y0 + r;
            const uint32_t cfg = cfg_from_masks(mk[t], mk[t + 1], mk1[t], mk1[t + 1], r);
            const bool l2 = needs_lut2(vol, g, tab, cfg, mk, mk1, t, r, x, y, k);
            const uint32_t info = owned_info_global(vol, g, x, y, k);
            const uint32_t nv = nvert_of(tab, cfg, l2) + __popc(info & 7u);
            const uint32_t nq = quad_count(info, cfg, x, y, k, g.cells, &n_drop);
            atomicAdd(&s_rv[r], nv);
            if (nq) atomicAdd(&s_rq[r], nq);
            ++n_act; n_l2 += l2;
        }
        __syncthreads();
        if (t < ROWS && y0 + t < g.cells.y) seg_cnt[seg_index(g, k, y0 + t, xs)] = make_uint2(s_rv[t], s_rq[t]);
    }
    if (n_act) atomicAdd(&s_stat[0], n_act);
    if (n_l2) atomicAdd(&s_stat[1], n_l2);
    if (n_drop) atomicAdd(&s_stat[2], n_drop);
    __syncthreads();
    if (t < 3 && s_stat[t]) atomicAdd(&counters[t], (unsigned long long)s_stat[t]);
}

// ---------------------------------------------------------------------------
// segment scan (decoupled look-back)

__global__ void __launch_bounds__(SCAN_NT) seg_scan(const uint2 *__restrict__ cnt, uint64_t n, ScanCtl ctl,
                                                    uint2 *__restrict__ off)
{
    __shared__ uint32_t s_slot;
    __shared__ unsigned long long s_warp[SCAN_NT / 32 + 1];
    __shared__ unsigned long long s_ex[2];
    const uint32_t tile = claim_tile(ctl.ticket, &s_slot);
    const uint64_t first = (uint64_t)tile * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
    uint2 c[SCAN_ITEMS];
    uint32_t sv = 0, sq = 0;
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        c[i] = first + i < n ? cnt[first + i] : make_uint2(0, 0);
        sv += c[i].x; sq += c[i].y;
    }
    unsigned long long tot;
    unsigned long long ex = block_exclusive_scan<SCAN_NT>((unsigned long long)sv | ((unsigned long long)sq << 32), s_warp, &tot);
    tile_prefix(ctl, tile, (uint32_t)tot, (uint32_t)(tot >> 32), s_ex);
    unsigned long long bv = s_ex[0] + (uint32_t)ex, bq = s_ex[1] + (uint32_t)(ex >> 32);
#pragma unroll
    for (int i = 0; i < SCAN_ITEMS; ++i) {
        if (first + i < n) off[first + i] = make_uint2((uint32_t)bv, (uint32_t)bq);
        bv += c[i].x; bq += c[i].y;
    }
}

// ---------------------------------------------------------------------------
// emit sweep

struct EmitSmem {
    uint64_t mask[2][W + 2];
    uint32_t dense[2][HROWS][HCOLS];     // per cell: vrel 11 | qrel 10 | cfg 8 | lut2 1  (active cells only)
    uint16_t list[2][MAXL];              // active cells in output order: row << 9 | col
    uint32_t nlist[2];
    uint32_t ball[NW][HROWS];            // per warp, per row: active lanes
    uint32_t rowstart[HROWS + 1];        // list index of each row's first entry
    uint32_t warpbase[NW][HROWS];        // list index of warp w's first entry in row r
    uint64_t halo_act;                   // active rows of the halo column
    uint32_t segv[2][HROWS][2];          // vertex offset of (row, own segment / next segment)
    uint32_t segq[2][HROWS];             // quad offset of (row, own segment)
    uint32_t rowbase_v[HROWS], rowbase_q[HROWS];
    uint8_t nvq[MAXL];                   // per list entry: nv | nq << 4
    unsigned long long scan_warp[NW + 1];
};

__device__ __forceinline__ uint32_t pack_cell(uint32_t vrel, uint32_t qrel, uint32_t cfg, bool l2)
{
    return vrel | (qrel << 11) | (cfg << 21) | ((l2 ? 1u : 0u) << 29);
}
__device__ __forceinline__ uint32_t cell_vrel(uint32_t p) { return p & 0x7ffu; }
__device__ __forceinline__ uint32_t cell_qrel(uint32_t p) { return (p >> 11) & 0x3ffu; }
__device__ __forceinline__ uint32_t cell_cfg(uint32_t p) { return (p >> 21) & 0xffu; }
__device__ __forceinline__ bool cell_l2(uint32_t p) { return (p >> 29) & 1u; }

template <class T>
__global__ void __launch_bounds__(NT) brick_emit(const T *__restrict__ vol, Geom g, const DeviceTables *__restrict__ tabp,
                                                 const uint2 *__restrict__ seg_off, float *__restrict__ verts, uint64_t vcap,
                                                 uint32_t *__restrict__ quads, uint64_t qcap, uint32_t *__restrict__ tris,
                                                 uint32_t *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    EmitSmem &S = *reinterpret_cast<EmitSmem *>(smem_raw);
    const DeviceTables &tab = *tabp;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t xs = blockIdx.x, yb = blockIdx.y, zb = blockIdx.z;
    const uint32_t x0 = xs * W, y0 = yb * ROWS, z0 = zb * g.zc;
    const uint32_t z1 = min(z0 + g.zc, g.cells.z);             // own planes [z0, z1)
    const uint32_t zlast = min(z1, g.cells.z - 1);             // classified planes [z0, zlast]
    const uint64_t hrowmask = row_valid_mask(y0, g.cells.y, HROWS);
    const bool colok = x0 + t < g.cells.x;
    const bool halo_col_ok = x0 + W < g.cells.x;

    load_masks(vol, g, x0, y0, z0, S.mask[z0 & 1]);
    for (uint32_t k = z0; k <= zlast; ++k) {
        const int cur = k & 1, prv = cur ^ 1;
        load_masks(vol, g, x0, y0, k + 1, S.mask[(k + 1) & 1]);
        // segment offsets of this plane's rows
        if (t < HROWS) {
            const uint32_t y = y0 + t;
            uint2 own = make_uint2(0, 0), nxt = make_uint2(0, 0);
            if (y < g.cells.y) {
                own = seg_off[seg_index(g, k, y, xs)];
                if (xs + 1 < g.nxs) nxt = seg_off[seg_index(g, k, y, xs + 1)];
            }
            S.segv[cur][t][0] = own.x; S.segv[cur][t][1] = nxt.x; S.segq[cur][t] = own.y;
        }
        __syncthreads();
        const uint64_t *mk = S.mask[cur], *mk1 = S.mask[(k + 1) & 1];
        // 1. activity of own column t (rows 0..32) and of the halo column
        const uint64_t act = colok ? active_rows(mk[t], mk[t + 1], mk1[t], mk1[t + 1]) & hrowmask : 0ull;
        if (t == 0)
            S.halo_act = halo_col_ok ? active_rows(mk[W], mk[W + 1], mk1[W], mk1[W + 1]) & hrowmask : 0ull;
#pragma unroll 1
        for (int r = 0; r < HROWS; ++r) {
            uint32_t b = __ballot_sync(0xffffffffu, (act >> r) & 1ull);
            if (lane == 0) S.ball[warp][r] = b;
        }
        __syncthreads();
        // 2. list layout: rows in order, within a row warps in order, halo column last
        if (warp == 0) {
            uint32_t run = 0;
            for (int r0 = 0; r0 < HROWS; r0 += 32) {
                const int r = r0 + lane;
                uint32_t cnt = 0;
                if (r < HROWS) {
                    for (int w = 0; w < NW; ++w) cnt += __popc(S.ball[w][r]);
                    cnt += (uint32_t)((S.halo_act >> r) & 1ull);
                }
                uint32_t inc = cnt;
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += y;
                }
                if (r < HROWS) {
                    uint32_t start = run + inc - cnt;
                    S.rowstart[r] = start;
                    for (int w = 0; w < NW; ++w) { S.warpbase[w][r] = start; start += __popc(S.ball[w][r]); }
                }
                run += __shfl_sync(0xffffffffu, inc, 31);
            }
            if (lane == 0) { S.rowstart[HROWS] = run; S.nlist[cur] = run; }
        }
        __syncthreads();
        // 3. scatter entries into the list
        {
            uint64_t a = act;
            const uint32_t lt = (1u << lane) - 1u;
            while (a) {
                const int r = __ffsll((long long)a) - 1;
                a &= a - 1;
                const uint32_t pos = S.warpbase[warp][r] + __popc(S.ball[warp][r] & lt);
                S.list[cur][pos] = (uint16_t)((r << 9) | t);
            }
            if (t == 0) {
                uint64_t h = S.halo_act;
                while (h) {
                    const int r = __ffsll((long long)h) - 1;
                    h &= h - 1;
                    S.list[cur][S.rowstart[r + 1] - 1] = (uint16_t)((r << 9) | W);
                }
            }
        }
        __syncthreads();
        // 4. per entry: config, LUT choice, counts (contiguous chunk per thread)
        const uint32_t L = S.nlist[cur];
        const uint32_t per = (L + NT - 1) / NT;
        const uint32_t e0 = min(L, per * t), e1 = min(L, e0 + per);
        uint32_t sv = 0, sq = 0;
        for (uint32_t e = e0; e < e1; ++e) {
            const uint32_t ent = S.list[cur][e];
            const int r = ent >> 9, c = ent & 0x1ff;
            const uint32_t x = x0 + c, y = y0 + r;
            const uint32_t cfg = cfg_from_masks(mk[c], mk[c + 1], mk1[c], mk1[c + 1], r);
            const bool l2 = needs_lut2(vol, g, tab, cfg, mk, mk1, c, r, x, y, k);
            const uint32_t info = owned_info_global(vol, g, x, y, k);
            const uint32_t nv = nvert_of(tab, cfg, l2) + __popc(info & 7u);
            uint32_t nq = 0, dummy = 0;
            if (r < ROWS && c < W) nq = quad_count(info, cfg, x, y, k, g.cells, &dummy);
            S.nvq[e] = (uint8_t)(nv | (nq << 4));
            S.dense[cur][r][c] = pack_cell(0, 0, cfg, l2);
            sv += nv; sq += nq;
        }
        unsigned long long tot;
        unsigned long long ex = block_exclusive_scan<NT>((unsigned long long)sv | ((unsigned long long)sq << 32), S.scan_warp, &tot);
        uint32_t pv = (uint32_t)ex, pq = (uint32_t)(ex >> 32);
        for (uint32_t e = e0; e < e1; ++e) {
            const uint32_t ent = S.list[cur][e];
            const int r = ent >> 9;
            if (e == S.rowstart[r]) { S.rowbase_v[r] = pv; S.rowbase_q[r] = pq; }
            const uint32_t b = S.nvq[e];
            pv += b & 15u; pq += b >> 4;
        }
        __syncthreads();
        pv = (uint32_t)ex; pq = (uint32_t)(ex >> 32);
        for (uint32_t e = e0; e < e1; ++e) {
            const uint32_t ent = S.list[cur][e];
            const int r = ent >> 9, c = ent & 0x1ff;
            uint32_t vrel = pv - S.rowbase_v[r], qrel = pq - S.rowbase_q[r];
            if (c == W) vrel = 0;                 // first cell of the next segment
            uint32_t &d = S.dense[cur][r][c];
            d = pack_cell(vrel, qrel, cell_cfg(d), cell_l2(d));
            const uint32_t b = S.nvq[e];
            pv += b & 15u; pq += b >> 4;
        }
        __syncthreads();
        // 5. vertices of own cells of plane k
        if (k < z1) {
            for (uint32_t e = e0; e < e1; ++e) {
                const uint32_t ent = S.list[cur][e];
                const int r = ent >> 9, c = ent & 0x1ff;
                if (r >= ROWS || c >= W) continue;
                const uint32_t x = x0 + c, y = y0 + r;
                const uint32_t d = S.dense[cur][r][c];
                const uint32_t cfg = cell_cfg(d);
                const bool l2 = cell_l2(d);
                const uint64_t vb = (uint64_t)S.segv[cur][r][0] + cell_vrel(d);
                const uint32_t nv = S.nvq[e] & 15u;
                if (vb + nv > vcap) { atomicOr(err, DEV_ERR_OVERFLOW); continue; }
                float v[8];
                v[0] = sample_at(vol, g, x, y, k);         v[1] = sample_at(vol, g, x + 1, y, k);
                v[2] = sample_at(vol, g, x + 1, y + 1, k); v[3] = sample_at(vol, g, x, y + 1, k);
                v[4] = sample_at(vol, g, x, y, k + 1);     v[5] = sample_at(vol, g, x + 1, y, k + 1);
                v[6] = sample_at(vol, g, x + 1, y + 1, k + 1); v[7] = sample_at(vol, g, x, y + 1, k + 1);
                const uint32_t info = owned_edge_info(v, g.iso);
                const uint32_t niso = nvert_of(tab, cfg, l2);
                Geo geo = cell_geo(x, y, k, g.cells, g.rng, g.mn);
                dual_vertices(tab, v, geo, g.iso, cfg, l2, x, y, k, niso, verts + 3 * vb);
                owned_edge_vertices(v, geo, g.iso, info, verts + 3 * (vb + niso));
            }
        }
        // 6. quads of own cells of plane k-1 (their +z ring cells are in plane k)
        if (k > z0) {
            const uint32_t kp = k - 1;
            const uint32_t Lp = S.nlist[prv];
            const uint32_t perp = (Lp + NT - 1) / NT;
            const uint32_t f0 = min(Lp, perp * t), f1 = min(Lp, f0 + perp);
            for (uint32_t e = f0; e < f1; ++e) {
                const uint32_t ent = S.list[prv][e];
                const int r = ent >> 9, c = ent & 0x1ff;
                if (r >= ROWS || c >= W) continue;
                const uint32_t x = x0 + c, y = y0 + r;
                const uint32_t d = S.dense[prv][r][c];
                const uint32_t cfg = cell_cfg(d);
                const uint32_t info = owned_info_global(vol, g, x, y, kp);
                uint64_t q = (uint64_t)S.segq[prv][r] + cell_qrel(d);
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, kp, g.cells) || !owned_sign_change(cfg, s)) continue;
                    if (q >= qcap) { atomicOr(err, DEV_ERR_OVERFLOW); break; }
                    const bool ccw = (info >> (s + 3)) & 1u;
                    uint32_t idx[4];
#pragma unroll
                    for (int it = 0; it < 4; ++it) {
                        const int kk = ccw ? it : (4 - it) & 3;
                        int re, dx, dy, dz;
                        ring_entry(s, kk, re, dx, dy, dz);
                        const int rr = r + dy, rc = c + dx, pl = dz ? cur : prv;
                        const uint32_t rd = S.dense[pl][rr][rc];
                        uint32_t m = lut_m(tab, cell_cfg(rd), cell_l2(rd), re);
                        if (m == 0xffu) { atomicOr(err, DEV_ERR_BOUNDS); m = 0; }
                        idx[it] = S.segv[pl][rr][rc == W ? 1 : 0] + cell_vrel(rd) + m;
                    }
                    reinterpret_cast<uint4 *>(quads)[q] = make_uint4(idx[0], idx[1], idx[2], idx[3]);
                    if (tris) {
                        uint32_t *tp = tris + 6 * q;
                        tp[0] = idx[0]; tp[1] = idx[1]; tp[2] = idx[2];
                        tp[3] = idx[2]; tp[4] = idx[3]; tp[5] = idx[0];
                    }
                    ++q;
                }
            }
        }
        __syncthreads();
    }
    // quads of the last own plane when it is the last plane of the volume
    // (only edge-6 quads remain; their ring stays in that plane)
    if (z1 == g.cells.z && zlast + 1 == z1) {
        const uint32_t kp = zlast;
        const int prv = kp & 1;
        const uint32_t Lp = S.nlist[prv];
        const uint32_t perp = (Lp + NT - 1) / NT;
        const uint32_t f0 = min(Lp, perp * t), f1 = min(Lp, f0 + perp);
        for (uint32_t e = f0; e < f1; ++e) {
            const uint32_t ent = S.list[prv][e];
            const int r = ent >> 9, c = ent & 0x1ff;
            if (r >= ROWS || c >= W) continue;
            const uint32_t x = x0 + c, y = y0 + r;
            const uint32_t d = S.dense[prv][r][c];
            const uint32_t cfg = cell_cfg(d);
            const uint32_t info = owned_info_global(vol, g, x, y, kp);
            uint64_t q = (uint64_t)S.segq[prv][r] + cell_qrel(d);
            if (!(info & 1u) || !owned_quad_in_volume(0, x, y, kp, g.cells) || !owned_sign_change(cfg, 0)) continue;
            if (q >= qcap) { atomicOr(err, DEV_ERR_OVERFLOW); continue; }
            const bool ccw = (info >> 3) & 1u;
            uint32_t idx[4];
#pragma unroll
            for (int it = 0; it < 4; ++it) {
                const int kk = ccw ? it : (4 - it) & 3;
                int re, dx, dy, dz;
                ring_entry(0, kk, re, dx, dy, dz);
                const int rr = r + dy, rc = c + dx;
                const uint32_t rd = S.dense[prv][rr][rc];
                uint32_t m = lut_m(tab, cell_cfg(rd), cell_l2(rd), re);
                if (m == 0xffu) { atomicOr(err, DEV_ERR_BOUNDS); m = 0; }
                idx[it] = S.segv[prv][rr][rc == W ? 1 : 0] + cell_vrel(rd) + m;
            }
            reinterpret_cast<uint4 *>(quads)[q] = make_uint4(idx[0], idx[1], idx[2], idx[3]);
            if (tris) {
                uint32_t *tp = tris + 6 * q;
                tp[0] = idx[0]; tp[1] = idx[1]; tp[2] = idx[2];
                tp[3] = idx[2]; tp[4] = idx[3]; tp[5] = idx[0];
            }
        }
    }
}

}  // namespace brick

// ---------------------------------------------------------------------------
// host side

bool brick_supports(const ExtractArgs &a)
{
    // 32-bit point indices per axis; at least one cell
    return a.cells.x >= 1 && a.cells.y >= 1 && a.cells.z >= 1;
}

template <class T>
static dmc_status brick_run_t(Ctx *ctx, const T *vol, const ExtractArgs &a, cudaStream_t st)
{
    using namespace brick;
    Geom g;
    g.pts = a.pts; g.cells = a.cells; g.iso = a.iso; g.mn = a.mn; g.rng = a.rng;
    g.nxs = (a.cells.x + W - 1) / W;
    g.nyb = (a.cells.y + ROWS - 1) / ROWS;
    g.zc = ZC;
    g.nzc = (a.cells.z + ZC - 1) / ZC;
    if (g.nyb > 65535 || g.nzc > 65535) return DMC_ERR_UNSUPPORTED;
    const uint64_t nseg = (uint64_t)a.cells.z * a.cells.y * g.nxs;
    const uint64_t n_tiles64 = (nseg + SCAN_TILE - 1) / SCAN_TILE;
    if (n_tiles64 >= (1ull << 31)) return DMC_ERR_UNSUPPORTED;
    const uint32_t n_tiles = (uint32_t)n_tiles64;
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    const size_t o_cnt = carve(8 * nseg), o_off = carve(8 * nseg), o_tiles = carve(sizeof(TileState) * n_tiles);
    dmc_status s = ctx_reserve_scratch(ctx, off);
    if (s != DMC_OK) return s;
    uint8_t *base = (uint8_t *)ctx->scratch;
    uint2 *seg_cnt = (uint2 *)(base + o_cnt), *seg_off = (uint2 *)(base + o_off);
    TileState *tiles = (TileState *)(base + o_tiles);

    CUDA_TRY(cudaMemsetAsync(tiles, 0, sizeof(TileState) * n_tiles, st));
    CUDA_TRY(cudaMemsetAsync(ctx->d_ctl, 0, sizeof(DevCtl), st));
    const dim3 grid(g.nxs, g.nyb, g.nzc);
    brick_count<T><<<grid, NT, 0, st>>>(vol, g, ctx->d_tab, seg_cnt, ctx->d_ctl->counters);
    ScanCtl ctl;
    ctl.tiles = tiles; ctl.ticket = &ctx->d_ctl->ticket; ctl.err = &ctx->d_ctl->err;
    ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = n_tiles;
    seg_scan<<<n_tiles, SCAN_NT, 0, st>>>(seg_cnt, nseg, ctl, seg_off);
    CUDA_TRY(cudaGetLastError());
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
    const size_t smem = sizeof(EmitSmem);
    CUDA_TRY(cudaFuncSetAttribute(brick_emit<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    brick_emit<T><<<grid, NT, smem, st>>>(vol, g, ctx->d_tab, seg_off, a.verts, a.vcap, a.quads, a.qcap, a.tris,
                                          &ctx->d_ctl->err);
    CUDA_TRY(cudaGetLastError());
    return DMC_OK;
}

dmc_status brick_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st)
{
    if (a.dtype == DMC_F32) return brick_run_t<float>(ctx, (const float *)a.vol, a, st);
    return brick_run_t<uint16_t>(ctx, (const uint16_t *)a.vol, a, st);
}

}  // namespace dmc
