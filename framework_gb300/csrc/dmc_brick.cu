// Brick path: persistent warps sweep bricks of the volume along z.
//
// A brick is 128 cell columns x 32 cell rows x a run of z planes and belongs
// to one warp.  The count sweep keeps two bits per sample of every point
// plane, "below" and "at or below the isovalue", in 64-bit masks per column
// (rows 0..32), built from the samples: each lane loads four adjacent samples
// of a row at a time, 8 rows in flight, and compares them (two uint16 samples
// per word at once).  A cell's configuration is a few shifts on the masks of
// two columns in two planes, and activity for all rows of a column takes ~12
// bitwise operations, so only active cells (a few percent) take the per-cell
// path.  A 32x32 bit transpose turns the column masks into each row's active
// cells in x order.  The count sweep classifies them (configuration, 2B/3B
// test, own-edge bits) and keeps the result in a cell store, one record per
// active cell and a header of row starts per brick plane; the emit sweep
// reads the store back instead of classifying the cells again, so it never
// touches the masks.  Warps never wait for each other: there is no
// block-level barrier in the sweep.
//
// Output order is the reference's (ascending cell index, x fastest,
// utils.hpp:72), so the active cells of one plane, row and 128-column
// segment form one contiguous output range, a "segment" (k, j, xs).
//   count sweep : per segment (vertices, quads); the cell store
//   scan        : decoupled look-back over segments -> offsets
//   emit sweep  : lists each plane's cells from the store, writes vertex
//                 positions and quads at their final places.
// Quads reference the dual vertices of the +x, +y, +z neighbours
// (dmc.cu:1636-1664): the emit sweep also lists the first cell column of the
// next segment (its vertices start at that segment's offset) and the first
// row of the next brick (ranked inside its own segment), both from their own
// bricks' store slots, and writes the quads of plane k once plane k+1 has
// been listed.
#include "dmc_device.cuh"
#include "dmc_scan.cuh"
#include "dmc_internal.h"
#include <algorithm>
#include <new>
#include <vector>
#include <type_traits>

namespace dmc {

namespace brick {

constexpr int GROUPS = 4;                 // columns per lane, 32 apart
constexpr int W = 32 * GROUPS;            // cell columns per brick (= segment width)
constexpr int ROWS = 32;                  // own cell rows
constexpr int HROWS = ROWS + 1;           // with the halo row
constexpr int MAXL = HROWS * (W + 1);     // most active cells one plane of a brick can hold
constexpr int CAP = 256;                  // entries kept in shared memory per plane
constexpr int OVF = MAXL - CAP;           // entries per plane that spill to global scratch
constexpr int NWB_COUNT = 8;              // warps per block of the count sweep (independent): 3 blocks per SM at 80
                                          // registers (4 blocks at 64 spilled and ran 10% slower)
constexpr int NWB_EMIT = 8;               // of the emit sweep: 3 blocks per SM
constexpr int nwb(bool emit) { return emit ? NWB_EMIT : NWB_COUNT; }
constexpr int kMaxSlabs = 32;             // z slabs of a streamed host extraction
constexpr int kTickets = 4 + 3 * kMaxSlabs; // work tickets: 4 for a batch, 3 per streamed slab
constexpr int QCAP = 256;                 // quad items of a plane kept in shared memory
constexpr int QOVF = 3 * W * ROWS - QCAP; // quad items of a plane that spill to global scratch
constexpr int SCAN_NT = 512, SCAN_ITEMS = 16, SCAN_TILE = SCAN_NT * SCAN_ITEMS;  // 8192 segments per tile: a short look-back chain
// a segment's count packs its vertices (at most 7 per cell) and quads (3) in 16 bits each; a thread's items add in place
static_assert(SCAN_ITEMS * 7 * W < 65536 && SCAN_ITEMS * 3 * W < 65536, "packed segment counts must not carry between halves");

// One volume of an extraction (a plain call has one, a batch many).
struct Geom {
    const void *data;
    uint3 pts, cells;
    uint32_t nxs, nyb, nzb, zc;
    uint64_t brick_base;   // first brick of this volume in the launch's brick numbering
    uint64_t seg_base;     // first segment of this volume in the shared segment arrays
    uint64_t nseg;
    uint64_t cell_base;    // first word of this volume's slots in the cell store
    float iso;
    uint32_t iso_u16;      // uint16 samples: v < iso  <=>  v < iso_u16 (65536: always)
    uint32_t isole_u16;    // uint16 samples: v <= iso <=>  v < isole_u16
    float3 mn, rng;
    const float *coord;    // point coordinates: x[0..cx], y[0..cy], z[0..cz]
    uint32_t vbase, qbase; // first vertex / quad of this volume in the output (set after the scan)
    uint32_t item;         // position of the volume in the caller's list
};

struct alignas(16) PlaneMasks {
    uint64_t lt[W + 2];                // bit r: sample (x0+c, y0+r) < iso
};

// Cell store (global scratch).  For every cell plane of every brick (a
// "slot": 128 columns x 32 rows of one plane) the count sweep writes what it
// found, and the emit sweep reads it back instead of classifying the cells
// again:
//   header (kHdrWords words): the first list entry of each row, rowstart[0..33]
//     as 16-bit pairs (rowstart[32] = entries of the slot), then the rows whose
//     cell in column 0 is active (bit r);
//   records (kRecWords words, one per active cell, row-major, x ascending):
//     column | row << 7 | config << 12 | LUT2 << 20 | own-edge info << 21.
// Slot s = (k * nyb + yb) * nxs + xs of a volume; its headers come first, then
// its records, 4 bytes per cell of the volume's bricks.
constexpr uint32_t kHdrWords = 20;
constexpr uint32_t kRecWords = W * ROWS;
__device__ __forceinline__ uint64_t cell_slot(const Geom &g, uint32_t k, uint32_t yb, uint32_t xs)
{
    return ((uint64_t)k * g.nyb + yb) * g.nxs + xs;
}
__device__ __forceinline__ uint32_t *slot_hdr(uint32_t *cells, const Geom &g, uint64_t s)
{
    return cells + g.cell_base + s * kHdrWords;
}
__device__ __forceinline__ uint32_t *slot_rec(uint32_t *cells, const Geom &g, uint64_t s)
{
    return cells + g.cell_base + (uint64_t)g.cells.z * g.nyb * g.nxs * kHdrWords + s * kRecWords;
}
// 16-bit entry i of a slot header
__device__ __forceinline__ uint32_t hdr_u16(const uint32_t *h, uint32_t i)
{
    return (__ldg(h + (i >> 1)) >> (16 * (i & 1))) & 0xffffu;
}
__device__ __forceinline__ uint32_t rec_pack(uint32_t c, uint32_t r, uint32_t cfg, bool l2, uint32_t info)
{
    return c | (r << 7) | (cfg << 12) | ((l2 ? 1u : 0u) << 20) | (info << 21);
}
__device__ __forceinline__ uint32_t rec_col(uint32_t w) { return w & 0x7fu; }
__device__ __forceinline__ uint32_t rec_row(uint32_t w) { return (w >> 7) & 0x1fu; }
__device__ __forceinline__ uint32_t rec_cfg(uint32_t w) { return (w >> 12) & 0xffu; }
__device__ __forceinline__ bool rec_l2(uint32_t w) { return (w >> 20) & 1u; }
__device__ __forceinline__ uint32_t rec_info(uint32_t w) { return (w >> 21) & 0x3fu; }

// Per-warp ranking state of both sweeps: each plane's active cells in list
// (output) order and per row.
struct alignas(16) RankSmem {
    uint32_t xrow[2][HROWS][GROUPS];   // per row: active cells in x order, word q = columns 32q..32q+31
    uint64_t hact[2];                  // halo column activity (bit = row)
    uint16_t rowstart[2][HROWS + 1];   // first list entry of each row
    uint32_t rowbase[HROWS];           // running (v | q << 16) prefix at each row start
    uint16_t lst0[CAP];                // list of plane slot 0: row << 8 | col (the count sweep uses only this)
};

// Per-warp state of the count sweep: the two point planes as bit masks.
struct alignas(16) CountSmem : RankSmem {
    PlaneMasks mask[2];                // point planes by parity
    uint32_t rowtot[ROWS];             // per-row (v | q << 16)
};

// Per-warp state of the emit sweep (no masks: it reads the cell store).
struct alignas(16) EmitSmem : RankSmem {
    uint16_t lst1[CAP];                // list of plane slot 1
    uint32_t segv[2][HROWS][2];        // vertex offset of (row, own / next segment)
    uint32_t segq[2][HROWS];           // quad offset of (row, own segment)
    uint16_t qitem[2][QCAP];           // the plane's quads in order: owner's list entry | owned edge << 13
    uint32_t qn[2];                    // quads of the plane
    uint32_t ent[2][CAP];              // a cell's record, then (once classified) its packed cell: vrel 11 | qrel 10 | cfg 8 | lut2 1
    uint8_t info[2][CAP];              // own-edge bipolar/ccw bits
};

static_assert(sizeof(EmitSmem) % 16 == 0 && sizeof(CountSmem) % 16 == 0, "per-warp shared memory must keep 16-byte alignment");

// shared memory layout of a sweep block: tables, then one per-warp state per warp
constexpr size_t kTablesBytes = (sizeof(DeviceTables) + 127) & ~(size_t)127;

struct Spill {                          // per warp slot, global memory
    uint32_t ent[2][OVF];
    uint16_t lst[2][OVF];
    uint8_t info[2][OVF];
    uint16_t qitem[2][QOVF];
};

// A plane's entries: the first CAP in shared memory, the rest in the warp's
// global spill slot.  Separate shared and global accesses (rather than one
// reference that may point to either) keep the common case on shared-memory
// instructions.  The count sweep has one list slot and no entry words.
template <class SM>
struct WarpMem {
    SM *s;
    Spill *g;
    __device__ __forceinline__ uint16_t *lst_s(int p) const
    {
        if constexpr (std::is_same<SM, EmitSmem>::value) return p ? s->lst1 : s->lst0;
        else return s->lst0;
    }
    __device__ __forceinline__ uint32_t ent(int p, uint32_t i) const
    {
        uint32_t v;
        if (i < CAP) v = s->ent[p][i]; else v = g->ent[p][i - CAP];
        return v;
    }
    __device__ __forceinline__ void set_ent(int p, uint32_t i, uint32_t v)
    {
        if (i < CAP) s->ent[p][i] = v; else g->ent[p][i - CAP] = v;
    }
    __device__ __forceinline__ uint32_t lst(int p, uint32_t i) const
    {
        uint32_t v;
        if (i < CAP) v = lst_s(p)[i]; else v = g->lst[p][i - CAP];
        return v;
    }
    __device__ __forceinline__ void set_lst(int p, uint32_t i, uint32_t v)
    {
        if (i < CAP) lst_s(p)[i] = (uint16_t)v; else g->lst[p][i - CAP] = (uint16_t)v;
    }
    __device__ __forceinline__ uint32_t info(int p, uint32_t i) const
    {
        uint32_t v;
        if (i < CAP) v = s->info[p][i]; else v = g->info[p][i - CAP];
        return v;
    }
    __device__ __forceinline__ void set_info(int p, uint32_t i, uint32_t v)
    {
        if (i < CAP) s->info[p][i] = (uint8_t)v; else g->info[p][i - CAP] = (uint8_t)v;
    }
    __device__ __forceinline__ uint32_t qitem(int p, uint32_t t) const
    {
        uint32_t v;
        if (t < QCAP) v = s->qitem[p][t]; else v = g->qitem[p][t - QCAP];
        return v;
    }
    __device__ __forceinline__ void set_qitem(int p, uint32_t t, uint32_t v)
    {
        if (t < QCAP) s->qitem[p][t] = (uint16_t)v; else g->qitem[p][t - QCAP] = (uint16_t)v;
    }
};

__device__ __forceinline__ uint64_t seg_index(const Geom &g, uint32_t k, uint32_t j, uint32_t xs)
{
    return g.seg_base + ((uint64_t)k * g.cells.y + j) * g.nxs + xs;
}

template <class T>
__device__ __forceinline__ float sample_at(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z)
{
    return load_sample(vol, ((uint64_t)z * g.pts.y + y) * g.pts.x + x);
}

template <class T>
__device__ __forceinline__ float sample_p(const T *vol, uint3 pts, uint32_t x, uint32_t y, uint32_t z)
{
    return load_sample(vol, ((uint64_t)z * pts.y + y) * pts.x + x);
}

// "below the isovalue" for a raw sample: float compare, or for uint16 the
// equivalent integer compare against the precomputed threshold
__device__ __forceinline__ uint32_t below(float v, float iso, uint32_t) { return v < iso ? 1u : 0u; }
__device__ __forceinline__ uint32_t below(uint16_t v, float, uint32_t thr) { return (uint32_t)v < thr ? 1u : 0u; }
__device__ __forceinline__ uint32_t at_or_below(float v, float iso, uint32_t) { return v <= iso ? 1u : 0u; }
__device__ __forceinline__ uint32_t at_or_below(uint16_t v, float, uint32_t thr) { return (uint32_t)v < thr ? 1u : 0u; }

template <class T>
__device__ __forceinline__ T raw_load(const T *p) { return __ldg(p); }

// Four consecutive samples in one load (8 bytes of uint16, 16 of float).
__device__ __forceinline__ uint2 load4(const uint16_t *p) { return __ldg(reinterpret_cast<const uint2 *>(p)); }
__device__ __forceinline__ float4 load4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
__device__ __forceinline__ uint16_t elem4(uint2 v, int q)
{
    const uint32_t w = q < 2 ? v.x : v.y;
    return (uint16_t)((q & 1) ? (w >> 16) : (w & 0xffffu));
}
__device__ __forceinline__ float elem4(float4 v, int q) { return q == 0 ? v.x : q == 1 ? v.y : q == 2 ? v.z : v.w; }

// Two uint16 samples per word (bits 0-15 and 16-31): bits 15 and 31 of the
// result say whether each is <= the matching half of m; mh = m | 0x80008000.
// (mh - (v & 0x7fff7fff)) cannot borrow across the halves, and its bit 15 of
// each half is (m >= v) over the low 15 bits; the top bits of m and v decide
// the rest.  Only bits 15 and 31 are meaningful.
__device__ __forceinline__ uint32_t le_u16x2(uint32_t v, uint32_t m, uint32_t mh)
{
    const uint32_t d = mh - (v & 0x7fff7fffu);
    return (m & ~v) | (~(m ^ v) & d);
}

// Column masks of point plane p for the lane's columns x0+lane+32j and the
// halo column x0+W: bit r = sample (x, y0+r, p) below the isovalue, rows
// 0..32 (the points of the brick's 32 cell rows).  Samples outside the volume read as 0 (their cells are never
// active).  Loads go out 8 rows per lane before their results are used; the
// next plane is not prefetched into L2 (all resident warps' planes together
// outrun the L2, and prefetched lines were evicted before their use, which
// read the volume 1.9 times instead of 1.35).  Only "below" is kept: where a
// sample equals the isovalue the active cells' corners are tested one by one
// (corner_eq4).
template <class T>
__device__ __noinline__ void load_plane(const T *vol, uint3 pts, float iso, uint32_t thr, uint32_t x0,
                                        uint32_t y0, uint32_t p, PlaneMasks &m, int lane)
{
    uint32_t lo[GROUPS] = {0, 0, 0, 0}, hi[GROUPS] = {0, 0, 0, 0};
    const bool pz = p < pts.z;
    const uint32_t nrow = pz ? min(33u, pts.y - y0) : 0u;
    // the halo column x0+W (rows lane and 32), loaded first so that its
    // latency overlaps the tile's rows
    float hv[1], hv2[1];
    bool hin[1], hin2[1];
#pragma unroll
    for (int hc = 0; hc < 1; ++hc) {
        const uint32_t x = x0 + W + hc;
        const bool okx = pz && x < pts.x;
        hin[hc] = okx && y0 + lane < pts.y;
        hin2[hc] = okx && lane < 1 && y0 + 32 + lane < pts.y;
        hv[hc] = hin[hc] ? sample_p(vol, pts, x, y0 + lane, p) : 0.f;
        hv2[hc] = hin2[hc] ? sample_p(vol, pts, x, y0 + 32 + lane, p) : 0.f;
    }
    const uint64_t sx = pts.x;
    const uint64_t plane0 = (uint64_t)p * pts.y;
    // Rows past the volume (or past 34) and columns past it give 0 bits: the
    // loads are predicated and the bits masked, so every brick takes the same
    // batched path (8 rows of loads in flight) whatever its position.
    const uint32_t rmask = nrow >= 32 ? 0xffffffffu : ((1u << nrow) - 1u);
    const uint32_t hmask = nrow > 32 ? ((1u << (nrow - 32)) - 1u) : 0u;
    uint32_t rmask_lt = rmask, hmask_lt = hmask;
    // All 128 columns in range and rows aligned for 4-sample loads
    // (warp-uniform): lane l takes the adjacent columns 4l..4l+3 of a row in
    // one load.  Otherwise lane l takes columns l, l+32, l+64, l+96.
    const bool vec = x0 + W <= pts.x && (pts.x & 3u) == 0 &&
                     (reinterpret_cast<uintptr_t>(vol) & (4 * sizeof(T) - 1)) == 0;
    if (vec) {
        const T *vb = vol + (plane0 + y0) * sx + x0 + 4 * lane;
        using V = decltype(load4(vb));
        if constexpr (std::is_same<T, uint16_t>::value) {
            // Two samples per 32-bit word, compared by le_u16x2 against t-1
            // (v < t <=> v <= t-1; t = 0 leaves nothing below).  Each row's
            // result bits (15 and 31) enter the accumulators from the top,
            // which shift right by one per row: after 16 rows, row j of the
            // half sits at bit j (even column) and 16+j (odd column).
            const uint32_t m_lt = (thr - 1u) & 0xffffu;
            const uint32_t M_lt = m_lt * 0x10001u;
            const uint32_t MH_lt = M_lt | 0x80008000u;
            if (thr == 0) rmask_lt = hmask_lt = 0;
#pragma unroll 1
            for (uint32_t h = 0; h < 2; ++h) {
                uint32_t ax = 0, ay = 0;   // columns (0,1) and (2,3)
#pragma unroll
                for (uint32_t r0 = 0; r0 < 16; r0 += 8) {
                    V v[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const uint32_t r = 16 * h + r0 + i;
                        v[i] = r < nrow ? load4(vb + (uint64_t)r * sx) : V{};
                    }
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        ax = (ax >> 1) | (le_u16x2(v[i].x, M_lt, MH_lt) & 0x80008000u);
                        ay = (ay >> 1) | (le_u16x2(v[i].y, M_lt, MH_lt) & 0x80008000u);
                    }
                }
                const uint32_t sh = 16 * h;
                lo[0] |= (ax & 0xffffu) << sh; lo[1] |= (ax >> 16) << sh;
                lo[2] |= (ay & 0xffffu) << sh; lo[3] |= (ay >> 16) << sh;
            }
            uint32_t ax = 0, ay = 0;      // rows 32, 33 end at bits 14, 15 (30, 31)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const V v = 32u + i < nrow ? load4(vb + (uint64_t)(32 + i) * sx) : V{};
                ax = (ax >> 1) | (le_u16x2(v.x, M_lt, MH_lt) & 0x80008000u);
                ay = (ay >> 1) | (le_u16x2(v.y, M_lt, MH_lt) & 0x80008000u);
            }
            hi[0] = (ax >> 14) & 3u; hi[1] = ax >> 30; hi[2] = (ay >> 14) & 3u; hi[3] = ay >> 30;
        } else {
#pragma unroll 1
            for (uint32_t r0 = 0; r0 < 32; r0 += 8) {
                V v[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) v[i] = r0 + i < nrow ? load4(vb + (uint64_t)(r0 + i) * sx) : V{};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int q = 0; q < 4; ++q) lo[q] |= below(elem4(v[i], q), iso, thr) << (r0 + i);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const V v = 32u + i < nrow ? load4(vb + (uint64_t)(32 + i) * sx) : V{};
#pragma unroll
                for (int q = 0; q < 4; ++q) hi[q] |= below(elem4(v, q), iso, thr) << i;
            }
        }
        // columns 4l..4l+3: two 16-byte stores
        const uint4 t0 = make_uint4(lo[0] & rmask_lt, hi[0] & hmask_lt, lo[1] & rmask_lt, hi[1] & hmask_lt);
        const uint4 t1 = make_uint4(lo[2] & rmask_lt, hi[2] & hmask_lt, lo[3] & rmask_lt, hi[3] & hmask_lt);
        uint4 *lt4 = reinterpret_cast<uint4 *>(&m.lt[4 * lane]);
        lt4[0] = t0; lt4[1] = t1;
    } else {
        const T *base = vol + (plane0 + y0) * sx + x0 + lane;
        bool cok[GROUPS];
#pragma unroll
        for (int j = 0; j < GROUPS; ++j) cok[j] = x0 + lane + 32 * j < pts.x;
#pragma unroll 1
        for (uint32_t r0 = 0; r0 < 32; r0 += 8) {
            T v[8][GROUPS];
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const T *row = base + (uint64_t)(r0 + i) * sx;
#pragma unroll
                for (int j = 0; j < GROUPS; ++j) v[i][j] = (r0 + i < nrow && cok[j]) ? raw_load(row + 32 * j) : T(0);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < GROUPS; ++j) lo[j] |= below(v[i][j], iso, thr) << (r0 + i);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const T *row = base + (uint64_t)(32 + i) * sx;
#pragma unroll
            for (int j = 0; j < GROUPS; ++j) {
                const T v = (32u + i < nrow && cok[j]) ? raw_load(row + 32 * j) : T(0);
                hi[j] |= below(v, iso, thr) << i;
            }
        }
#pragma unroll
        for (int j = 0; j < GROUPS; ++j) {
            const uint32_t cm = cok[j] ? 0xffffffffu : 0u;
            m.lt[lane + 32 * j] = (uint64_t)(lo[j] & rmask & cm) | ((uint64_t)(hi[j] & hmask & cm) << 32);
        }
    }
    {
        const uint32_t l32 = __ballot_sync(0xffffffffu, hin[0] && hv[0] < iso);
        const uint32_t h1 = __ballot_sync(0xffffffffu, hin2[0] && hv2[0] < iso) & 1u;
        if (lane == 0) { m.lt[W] = (uint64_t)l32 | ((uint64_t)h1 << 32); m.lt[W + 1] = 0; }
    }
}

// Corners 2, 5, 6, 7 of cell (x, y, z), for their at-the-isovalue bits
// (corner_eq4): where a sample equals the isovalue "at or below" differs from
// "below".  Read from the samples (a few active cells per brick plane)
// instead of keeping a second mask per sample.  Only corners that are not
// below the isovalue (their bit clear in the configuration) can equal it, so
// only those are read; the others get a NaN, which equals nothing.
struct Corners4 { float s2, s5, s6, s7; };

template <class T>
__device__ __forceinline__ Corners4 load_corners4(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z,
                                                  uint32_t cfg)
{
    const uint64_t sy = g.pts.x, sz = (uint64_t)g.pts.x * g.pts.y;
    const T *p = vol + (uint64_t)z * sz + (uint64_t)y * sy + x;
    const float none = __int_as_float(0x7fc00000);
    return Corners4{(cfg >> 2) & 1u ? none : load_sample(p, sy + 1), (cfg >> 5) & 1u ? none : load_sample(p, sz + 1),
                    (cfg >> 6) & 1u ? none : load_sample(p, sz + sy + 1), (cfg >> 7) & 1u ? none : load_sample(p, sz + sy)};
}

// bit 0 corner 2, bit 1 corner 5, bit 2 corner 6, bit 3 corner 7: sample == iso
__device__ __forceinline__ uint32_t corner_eq4(const Corners4 &s, float iso)
{
    return (s.s2 == iso ? 1u : 0u) | (s.s5 == iso ? 2u : 0u) | (s.s6 == iso ? 4u : 0u) | (s.s7 == iso ? 8u : 0u);
}

// Reference bipolarity and ccw bits of the cell's own edges (dmc.cu:1199-1216)
// from the "below" (lt) and "at or below" (le) bits of corners 2, 5, 6, 7:
// ref_bipolar(a,b) = not both below, not both above, not both equal.
__device__ __forceinline__ uint32_t info_from_bits(uint32_t cfg, uint32_t le4)
{
    // le4: bit 0 corner 2, bit 1 corner 5, bit 2 corner 6, bit 3 corner 7
    const uint32_t l2 = (cfg >> 2) & 1u, l5 = (cfg >> 5) & 1u, l6 = (cfg >> 6) & 1u, l7 = (cfg >> 7) & 1u;
    const uint32_t e2 = le4 & 1u, e5 = (le4 >> 1) & 1u, e6 = (le4 >> 2) & 1u, e7 = (le4 >> 3) & 1u;
    const uint32_t q2 = e2 & ~l2, q5 = e5 & ~l5, q6 = e6 & ~l6, q7 = e7 & ~l7;   // exactly at the isovalue
    const uint32_t b6 = ~(l2 & l6) & (e2 | e6) & ~(q2 & q6) & 1u;
    const uint32_t b9 = ~(l5 & l6) & (e5 | e6) & ~(q5 & q6) & 1u;
    const uint32_t b10 = ~(l7 & l6) & (e7 | e6) & ~(q7 & q6) & 1u;
    return b6 | (b9 << 1) | (b10 << 2) | ((b6 & e2) << 3) | ((b9 & e5) << 4) | ((b10 & e7) << 5);
}

// le bits of corners 2, 5, 6, 7 of the cell in row r (masks of columns c, c+1
// in planes k (B: column c+1) and k+1 (C: column c, D: column c+1)).
__device__ __forceinline__ uint32_t le4_from_masks(uint64_t B, uint64_t C, uint64_t D, int r)
{
    return (uint32_t)((B >> (r + 1)) & 1u) | ((uint32_t)((D >> r) & 1u) << 1) |
           ((uint32_t)((D >> (r + 1)) & 1u) << 2) | ((uint32_t)((C >> (r + 1)) & 1u) << 3);
}

// Rows r (bit r) whose cell has corners on both sides (A,B: plane k columns
// c,c+1; C,D: plane k+1).
__device__ __forceinline__ uint64_t active_rows(uint64_t A, uint64_t B, uint64_t C, uint64_t D)
{
    const uint64_t a = A & B & C & D, o = A | B | C | D;
    return (o | (o >> 1)) & ~(a & (a >> 1));
}

// Configuration of the cell in row r (corner order of dmc.cu:1044-1054).
__device__ __forceinline__ uint32_t cfg_from_masks(uint64_t A, uint64_t B, uint64_t C, uint64_t D, int r)
{
    const uint32_t a = (uint32_t)(A >> r), b = (uint32_t)(B >> r), c = (uint32_t)(C >> r), d = (uint32_t)(D >> r);
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

// 2B/3B correction (dmc.cu:1232-1371): LUT2 when the config is one of the 36
// ambiguous ones and so is the face neighbour's.  The neighbour's config
// comes from the masks when it lies in the window (columns 0..W, rows 0..32,
// same plane), otherwise from eight global loads.
template <class T>
__device__ __forceinline__ bool needs_lut2(const T *vol, const Geom &g, const DeviceTables &tab, uint32_t cfg,
                                           const uint64_t *mk, const uint64_t *mk1, int c, int r,
                                           uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t face = tab.amb_face[cfg];
    if (face == 0xffu) return false;
    const int dir = tab.face_dir[face];
    const int dx = dir == 0 ? 1 : (dir == 1 ? -1 : 0);
    const int dy = dir == 2 ? 1 : (dir == 3 ? -1 : 0);
    const int dz = dir == 4 ? 1 : (dir == 5 ? -1 : 0);
    const long long nx = (long long)x + dx, ny = (long long)y + dy, nz = (long long)z + dz;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= g.cells.x || ny >= g.cells.y || nz >= g.cells.z) return false;
    uint32_t ncfg;
    const int nc = c + dx, nr = r + dy;
    if (dz == 0 && nc >= 0 && nc < W && nr >= 0 && nr < ROWS)
        ncfg = cfg_from_masks(mk[nc], mk[nc + 1], mk1[nc], mk1[nc + 1], nr);
    else
        ncfg = cfg_global(vol, g, (uint32_t)nx, (uint32_t)ny, (uint32_t)nz);
    return tab.amb_face[ncfg] != 0xffu;
}

// Owned edges (bit s: edge 6, 9, 10) whose quad the cell writes: bipolar by
// the reference's test, quad inside the volume, sign change in the config.
__device__ __forceinline__ uint32_t quad_want(uint32_t info, uint32_t cfg, uint32_t x, uint32_t y, uint32_t z, uint3 cells)
{
    uint32_t want = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s)
        if ((info & (1u << s)) && owned_quad_in_volume(s, x, y, z, cells) && owned_sign_change(cfg, s)) want |= 1u << s;
    return want;
}

__device__ __forceinline__ uint32_t quad_count(uint32_t info, uint32_t cfg, uint32_t x, uint32_t y, uint32_t z,
                                               uint3 cells, uint32_t &dropped)
{
    uint32_t nq = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        if (!(info & (1u << s)) || !owned_quad_in_volume(s, x, y, z, cells)) continue;
        if (owned_sign_change(cfg, s)) ++nq; else ++dropped;
    }
    return nq;
}

__device__ __forceinline__ uint32_t pack_cell(uint32_t vrel, uint32_t qrel, uint32_t cfg, bool l2)
{
    return vrel | (qrel << 11) | (cfg << 21) | ((l2 ? 1u : 0u) << 29);
}
__device__ __forceinline__ uint32_t cell_vrel(uint32_t p) { return p & 0x7ffu; }
__device__ __forceinline__ uint32_t cell_qrel(uint32_t p) { return (p >> 11) & 0x3ffu; }
__device__ __forceinline__ uint32_t cell_cfg(uint32_t p) { return (p >> 21) & 0xffu; }
__device__ __forceinline__ bool cell_l2(uint32_t p) { return (p >> 29) & 1u; }

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// 32x32 bit transpose across the warp: on entry lane l holds column l (bit r
// = row r); on exit lane r holds row r (bit l = column l).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, int lane)
{
    const uint32_t lo[5] = {0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        const int s = 16 >> i;
        const uint32_t y = __shfl_xor_sync(0xffffffffu, x, s);
        x = (lane & s) ? ((x & ~lo[i]) | ((y & ~lo[i]) >> s)) : ((x & lo[i]) | ((y & lo[i]) << s));
    }
    return x;
}

struct EmitOut {
    const uint2 *seg_off;
    float *verts; uint64_t vcap;
    uint32_t *quads; uint64_t qcap;
    uint32_t *tris;
};

// Device-resident plan of one pipeline launch (a plain call is a batch of
// one).  The host writes it to pinned memory and one copy moves it to the
// device, so the kernels take every batch-dependent size from here and a
// captured graph replays any batch that fits the scratch layout.
// Bricks [lo, lo + cnt) of a launch's numbering (cnt = kAllBricks: all of
// them).  The count sweep processes only cell planes below zlim (a sharded
// extraction counts the next shard's first plane this way), and with
// kNoStats adds nothing to the active / LUT2 / dropped-quad counters.
struct BrickRange {
    uint32_t lo, cnt;
    uint32_t zlim = 0xffffffffu;
    uint32_t flags = 0;
};
constexpr uint32_t kAllBricks = 0xffffffffu;
constexpr uint32_t kNoStats = 1u;

struct alignas(64) BatchHead {
    unsigned long long nbricks[2];   // bricks of the f32 / u16 volumes
    unsigned long long nseg;         // segments of all volumes
    uint32_t nvol[2];                // geoms[]: the f32 volumes, then the u16 ones
    uint32_t n;                      // volumes
    uint32_t n_tiles;                // scan tiles over nseg
};

__device__ __forceinline__ const Geom *batch_geoms(const BatchHead *h)
{
    return reinterpret_cast<const Geom *>(h + 1);
}

// Stage the lookup tables in shared memory (once per block; warps are persistent).
__device__ __forceinline__ const DeviceTables &stage_tables(const DeviceTables *g, DeviceTables *s)
{
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g);
    uint32_t *dst = reinterpret_cast<uint32_t *>(s);
    for (uint32_t i = threadIdx.x; i < sizeof(DeviceTables) / 4; i += blockDim.x) dst[i] = src[i];
    __syncthreads();
    return *s;
}

// Volume of launch brick bg: the last one whose first brick is <= bg.
__device__ __forceinline__ uint32_t volume_of(const Geom *vols, uint32_t nvols, uint64_t bg)
{
    uint32_t lo = 0, hi = nvols - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (vols[mid].brick_base <= bg) lo = mid; else hi = mid - 1;
    }
    return lo;
}

constexpr uint32_t kMaxRun = 16;   // most bricks one claim of the count sweep takes

// Count sweep work claim (guided self-scheduling): a run of consecutive units
// sized to about half of what remains per warp, between 1 and kMaxRun, so
// early claims are long (few halo planes) and the last ones short (even
// finish).  [lo, hi) is empty once every unit is taken.
__device__ __forceinline__ void claim_run(uint32_t *ticket, uint32_t n_units, uint32_t n_warps, int lane,
                                          uint32_t &lo, uint32_t &hi)
{
    uint32_t t = 0, r = 0;
    if (lane == 0) {
        const uint32_t seen = *reinterpret_cast<volatile uint32_t *>(ticket);
        const uint32_t want = n_units > seen ? (n_units - seen) / (2u * n_warps) : 0u;
        r = want < 1u ? 1u : (want > kMaxRun ? kMaxRun : want);
        t = atomicAdd(ticket, r);
    }
    t = __shfl_sync(0xffffffffu, t, 0);
    r = __shfl_sync(0xffffffffu, r, 0);
    lo = t;
    hi = t < n_units ? (n_units - t < r ? n_units : t + r) : t;
}

// Count sweep unit u of a launch, numbered z fastest within each column of
// bricks so that consecutive units are z neighbours: its column (xs + nxs *
// yb), z brick, and the units left in the column from it.  All bricks of a
// launch (u is the launch brick number; volumes keep their brick ranges), or
// a range of whole brick planes of one volume (u counts from its start).
__device__ __forceinline__ uint32_t count_unit(const Geom &g, const BrickRange &range, uint32_t u, uint32_t &zb,
                                               uint32_t &limit)
{
    const uint32_t ncol = g.nxs * g.nyb;
    if (range.cnt == kAllBricks) {
        const uint32_t b = (uint32_t)(u - g.brick_base);
        zb = b % g.nzb;
        limit = g.nzb - zb;
        return b / g.nzb;
    }
    const uint32_t zb_lo = (uint32_t)(((uint64_t)range.lo - g.brick_base) / ncol), nzr = range.cnt / ncol;
    zb = zb_lo + u % nzr;
    limit = nzr - u % nzr;
    return u / nzr;
}

// Corner samples 2, 5, 6, 7 (the cell's own edges) or all eight.
template <class T>
__device__ __forceinline__ void load_cell(const T *vol, const Geom &g, uint32_t x, uint32_t y, uint32_t z, float v[8],
                                          bool all)
{
    const uint64_t sy = g.pts.x, sz = (uint64_t)g.pts.x * g.pts.y;
    const T *p = vol + (uint64_t)z * sz + (uint64_t)y * sy + x;
    v[2] = load_sample(p, sy + 1);      v[5] = load_sample(p, sz + 1);
    v[6] = load_sample(p, sz + sy + 1); v[7] = load_sample(p, sz + sy);
    if (all) {
        v[0] = load_sample(p, 0);  v[1] = load_sample(p, 1);
        v[3] = load_sample(p, sy); v[4] = load_sample(p, sz);
    }
}

// Quad rings of owned edges 6, 9, 10 (dmc.cu:653-664), one byte per ring slot:
// bit 0 plane (0: k-1, 1: k), bits 1-2 base entry (0 own, 1 (c,r+1,k-1),
// 2 (c,r,k), 3 (c,r+1,k)), bit 3 next entry (+x neighbour), bit 4 row + 1.
constexpr uint32_t kRing6 = 0x121a0800u, kRing9 = 0x080d0500u, kRing10 = 0x05171200u;
// ring edges: e6 ring 6,7,4,5; e9 ring 9,1,3,11; e10 ring 10,8,0,2
__device__ __forceinline__ uint32_t ring_edge(int s, int kk)
{
    const unsigned long long E = 0x208ab3195476ull;   // 12 nibbles: s*4 + kk
    return (uint32_t)((E >> (4 * (4 * s + kk))) & 0xfull);
}

// Emit sweep, plane k of brick (xs, yb), from the cell store: lists the
// plane's cells in output order, with their packed cell words and own-edge
// bits, and writes the vertices of its own cells (for k < zv).  Besides the
// slot's own cells, the quads need the halo: column W (column 0 of the next x
// brick) and row 32 (row 0 of the next y brick).  List order is rows 0..31,
// each followed by its column-W cell, then row 32 and its column-W cell;
// xrow[p], hact[p] and rowstart[p][0..33] index the list, segv[p] / segq[p]
// hold the rows' segment offsets.  Each record is read and classified once:
// its counts, its place in its row (a segmented scan: records come row by
// row) and its vertices are taken in the same pass.  Returns the list length.
template <class T, class SM>
__device__ __forceinline__ uint32_t emit_plane(uint32_t *cells, const Geom &g, const T *vol, const DeviceTables &tab,
                                               const EmitOut &out, uint32_t *err, uint32_t k, uint32_t zv,
                                               uint32_t xs, uint32_t yb, int p, int lane, SM &S, WarpMem<SM> &M)
{
    const uint64_t s0 = cell_slot(g, k, yb, xs);
    const uint32_t x0 = xs * W, y0 = yb * ROWS;
    const bool hx = xs + 1 < g.nxs, hy = yb + 1 < g.nyb;
    // the rows' segment offsets, issued first (their latency overlaps the header)
    uint2 so0 = make_uint2(0, 0), sn0 = make_uint2(0, 0), so1 = make_uint2(0, 0), sn1 = make_uint2(0, 0);
    if (y0 + lane < g.cells.y) {
        so0 = out.seg_off[seg_index(g, k, y0 + lane, xs)];
        if (hx) sn0 = out.seg_off[seg_index(g, k, y0 + lane, xs + 1)];
    }
    if (lane == 0 && y0 + 32 < g.cells.y) {
        so1 = out.seg_off[seg_index(g, k, y0 + 32, xs)];
        if (hx) sn1 = out.seg_off[seg_index(g, k, y0 + 32, xs + 1)];
    }
    const uint32_t *h0 = slot_hdr(cells, g, s0);
    const uint32_t *r0 = slot_rec(cells, g, s0);
    // own rows: lane r holds the first entry of row r and of row r+1
    const uint32_t st = hdr_u16(h0, lane), en = hdr_u16(h0, lane + 1);
    const uint32_t lown = __shfl_sync(0xffffffffu, en, 31);
    if (lown == 0) {
        // No own cell: no quad of plane k-1 has a ring cell in this plane
        // (each ring around an owned edge 9 or 10 holds the cell above the
        // owner, in an own column and row), so the halo is not needed.
        S.rowstart[p][lane] = 0;
        *reinterpret_cast<uint4 *>(S.xrow[p][lane]) = make_uint4(0u, 0u, 0u, 0u);
        if (lane == 0) {
            S.rowstart[p][32] = 0;
            S.rowstart[p][33] = 0;
            S.hact[p] = 0;
            S.qn[p] = 0;
            *reinterpret_cast<uint4 *>(S.xrow[p][32]) = make_uint4(0u, 0u, 0u, 0u);
        }
        __syncwarp();
        return 0;
    }
    // segment offsets of the rows (loaded before the slot header was checked)
    S.segv[p][lane][0] = so0.x; S.segv[p][lane][1] = sn0.x; S.segq[p][lane] = so0.y;
    if (lane == 0) { S.segv[p][32][0] = so1.x; S.segv[p][32][1] = sn1.x; S.segq[p][32] = so1.y; }
    // halo column (the next x brick's rows with an active column-0 cell) and
    // the corner cell of row 32
    uint32_t col0 = 0, hxrec = 0, n32 = 0, corner = 0, crec = 0;
    if (hx) {
        const uint32_t *hX = slot_hdr(cells, g, s0 + 1);
        col0 = __ldg(hX + 17);
        if ((col0 >> lane) & 1u) hxrec = __ldg(slot_rec(cells, g, s0 + 1) + hdr_u16(hX, lane));
    }
    if (hy) {
        n32 = hdr_u16(slot_hdr(cells, g, s0 + g.nxs), 1);   // entries of row 0 of the next y brick
        if (hx && (__ldg(slot_hdr(cells, g, s0 + g.nxs + 1) + 17) & 1u)) {
            corner = 1;
            crec = __ldg(slot_rec(cells, g, s0 + g.nxs + 1));
        }
    }
    const uint32_t hcp = __popc(col0 & ((1u << lane) - 1u));   // halo entries in the rows before row lane
    const uint32_t start32 = lown + __popc(col0);
    const uint32_t L = start32 + n32 + corner;
    S.rowstart[p][lane] = (uint16_t)(st + hcp);
    *reinterpret_cast<uint4 *>(S.xrow[p][lane]) = make_uint4(0u, 0u, 0u, 0u);
    // column-W cells are the first of their segment (vertex offset 0)
    if (lane == 0) {
        S.rowstart[p][32] = (uint16_t)start32;
        S.rowstart[p][33] = (uint16_t)L;
        S.hact[p] = (uint64_t)col0 | ((uint64_t)corner << 32);
        *reinterpret_cast<uint4 *>(S.xrow[p][32]) = make_uint4(0u, 0u, 0u, 0u);
        if (corner) {
            M.set_lst(p, start32 + n32, (32u << 8) | W);
            M.set_ent(p, start32 + n32, pack_cell(0u, 0u, rec_cfg(crec), rec_l2(crec)));
            M.set_info(p, start32 + n32, rec_info(crec) & 0x38u);
        }
    }
    if ((col0 >> lane) & 1u) {   // last entry of row lane
        M.set_lst(p, en + hcp, ((uint32_t)lane << 8) | W);
        M.set_ent(p, en + hcp, pack_cell(0u, 0u, rec_cfg(hxrec), rec_l2(hxrec)));
        M.set_info(p, en + hcp, rec_info(hxrec) & 0x38u);
    }
    __syncwarp();
    // own cells, 32 at a time; each round's records are read one round ahead
    // (an L2 prefetch of the next round's corner lines, tried here, made the
    // sweep 3% slower)
    uint32_t run = 0;
    uint32_t nrec = (uint32_t)lane < lown ? __ldg(r0 + lane) : 0u;
    for (uint32_t b = 0; b < lown; b += 32) {
        const uint32_t i = b + lane;
        const bool valid = i < lown;
        const uint32_t rec = nrec;
        nrec = i + 32 < lown ? __ldg(r0 + i + 32) : 0u;
        const uint32_t r = rec_row(rec), c = rec_col(rec);
        const uint32_t shift = __shfl_sync(0xffffffffu, hcp, (int)r);
        const uint32_t first = __shfl_sync(0xffffffffu, st, (int)r);
        const uint32_t cfg = rec_cfg(rec), info = rec_info(rec);
        const bool l2 = rec_l2(rec);
        const uint32_t x = x0 + c, y = y0 + r;
        float v[8];
        if (valid && k < zv) load_cell(vol, g, x, y, k, v, true);
        uint32_t packed = 0, want = 0;
        if (valid) {
            want = quad_want(info, cfg, x, y, k, g.cells);
            packed = (nvert_of(tab, cfg, l2) + __popc(info & 7u)) | (__popc(want) << 16);
        }
        const uint32_t incl = warp_incl_scan(packed, lane);
        const uint32_t ex = run + incl - packed;
        run += __shfl_sync(0xffffffffu, incl, 31);
        if (valid && i == first) S.rowbase[r] = ex;
        __syncwarp();
        if (valid) {
            const uint32_t rb = S.rowbase[r];
            const uint32_t vrel = (ex & 0xffffu) - (rb & 0xffffu);
            const uint32_t qrel = (ex >> 16) - (rb >> 16);
            M.set_lst(p, i + shift, (r << 8) | c);
            M.set_ent(p, i + shift, pack_cell(vrel, qrel, cfg, l2));
            M.set_info(p, i + shift, want | (info & 0x38u));   // the quads need only these: wanted edges, ccw bits
            // the cell's quads, at their place among the plane's quads
            for (uint32_t w = want, t = ex >> 16; w; w &= w - 1, ++t)
                M.set_qitem(p, t, (i + shift) | ((uint32_t)(__ffs(w) - 1) << 13));
            atomicOr(&S.xrow[p][r][c >> 5], 1u << (c & 31));
            if (k < zv) {
                const uint32_t nv = packed & 0xffffu;
                const uint64_t vb = (uint64_t)S.segv[p][r][0] + vrel;
                if (vb + nv > out.vcap) {
                    atomicOr(err, DEV_ERR_OVERFLOW);
                } else {
                    Geo geo;
                    geo.x0 = g.coord[x]; geo.x1 = g.coord[x + 1];
                    geo.y0 = g.coord[g.pts.x + y]; geo.y1 = g.coord[g.pts.x + y + 1];
                    geo.z0 = g.coord[g.pts.x + g.pts.y + k]; geo.z1 = g.coord[g.pts.x + g.pts.y + k + 1];
                    cell_vertices(tab, v, geo, g.iso, cfg, l2, nvert_of(tab, cfg, l2), info, x, y, k,
                                  out.verts + 3 * vb);
                }
            }
        }
        __syncwarp();
    }
    if (lane == 0) S.qn[p] = run >> 16;
    // halo row (row 0 of the next y brick): its place in its own segment
    if (n32) {
        const uint32_t *rY = slot_rec(cells, g, s0 + g.nxs);
        uint32_t hrun = 0;
        for (uint32_t b = 0; b < n32; b += 32) {
            const uint32_t j = b + lane;
            const uint32_t rec = j < n32 ? __ldg(rY + j) : 0u;
            const uint32_t cfg = rec_cfg(rec), info = rec_info(rec), c = rec_col(rec);
            const bool l2 = rec_l2(rec);
            const uint32_t nv = j < n32 ? nvert_of(tab, cfg, l2) + __popc(info & 7u) : 0u;
            const uint32_t incl = warp_incl_scan(nv, lane);
            if (j < n32) {
                M.set_lst(p, start32 + j, (32u << 8) | c);
                M.set_ent(p, start32 + j, pack_cell(hrun + incl - nv, 0u, cfg, l2));
                M.set_info(p, start32 + j, info & 0x38u);
                atomicOr(&S.xrow[p][32][c >> 5], 1u << (c & 31));
            }
            hrun += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    __syncwarp();
    return L;
}

// One sweep kernel for both passes.
//   EMIT = false (count): ranks and classifies the active cells of the
//     brick's own 32 rows, writes per-segment (vertices, quads) totals and
//     each plane's slot of the cell store.
//   EMIT = true: reads each plane's slot (with the halo row and column from
//     the neighbouring slots), writes the vertices of plane k at their final
//     offsets and the quads of plane k-1.
// Active cells are compacted per plane in output order and processed 32 at a
// time, one per lane; quads are compacted the same way.
template <class T, bool EMIT>
__global__ void __launch_bounds__(32 * nwb(EMIT), 3) brick_sweep(const BatchHead *__restrict__ head, uint32_t group,
                                                                 BrickRange range, const DeviceTables *__restrict__ tabp,
                                                                 uint32_t *__restrict__ seg_cnt, EmitOut out,
                                                                 Spill *__restrict__ spill, uint32_t *__restrict__ cells,
                                                                 uint32_t *ticket, unsigned long long *counters,
                                                                 uint32_t *err)
{
    using SM = typename std::conditional<EMIT, EmitSmem, CountSmem>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (head->nbricks[group] == 0) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const DeviceTables &tab = stage_tables(tabp, reinterpret_cast<DeviceTables *>(smem_raw));
    SM &S = *reinterpret_cast<SM *>(smem_raw + kTablesBytes + (size_t)warp * sizeof(SM));
    WarpMem<SM> M{&S, spill + (uint64_t)blockIdx.x * nwb(EMIT) + warp};
    uint32_t n_act = 0, n_l2 = 0, n_drop = 0;
    const uint32_t nvols = head->nvol[group];
    const uint64_t nbricks = head->nbricks[group];
    const Geom *__restrict__ vols = batch_geoms(head) + (group ? head->nvol[0] : 0u);

    // Count sweep: the claimed bricks not yet swept, [span, span_end) in the
    // z-fastest numbering of count_unit.  It sweeps a run of bricks along z
    // of one column as one tall brick: the masks of a plane carry from one
    // brick to the next, so a run loads one plane more than it owns, not one
    // per brick.  The emit sweep claims single bricks in the launch's
    // numbering (x fastest): its work per brick is uneven, and concurrent
    // warps then gather from nearby planes (runs measured 14% slower there).
    uint32_t span = 0, span_end = 0;
    const uint32_t n_units = range.cnt == kAllBricks ? (uint32_t)nbricks : range.cnt;
    for (;;) {
        uint32_t vi, xs, yb, zb, zrun;
        if constexpr (EMIT) {
            uint32_t t = 0;
            if (lane == 0) t = atomicAdd(ticket, 1u);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= range.cnt) break;
            const uint64_t bg = (uint64_t)range.lo + t;
            if (bg >= nbricks) break;
            vi = volume_of(vols, nvols, bg);
            const uint32_t nxs = vols[vi].nxs, nyb = vols[vi].nyb;
            const uint32_t b = (uint32_t)(bg - vols[vi].brick_base);
            xs = b % nxs; yb = (b / nxs) % nyb; zb = b / (nxs * nyb);
            zrun = 1;
        } else {
            if (span >= span_end) {
                claim_run(ticket, n_units, gridDim.x * nwb(EMIT), lane, span, span_end);
                if (span >= span_end) break;
            }
            vi = volume_of(vols, nvols, range.cnt == kAllBricks ? (uint64_t)span : (uint64_t)range.lo);
            uint32_t limit;
            const uint32_t col = count_unit(vols[vi], range, span, zb, limit);
            zrun = min(limit, span_end - span);
            span += zrun;
            xs = col % vols[vi].nxs; yb = col / vols[vi].nxs;
        }
        const Geom g = vols[vi];
        const uint32_t z0 = zb * g.zc, z1 = min((zb + zrun) * g.zc, g.cells.z);
        const T *__restrict__ vol = reinterpret_cast<const T *>(g.data);
        const uint32_t x0 = xs * W, y0 = yb * ROWS;
        // the emit sweep also visits plane z1: quads of plane z1-1 reference it
        const uint32_t kend = EMIT ? z1 : min(z1, range.zlim) - 1;

        // Count sweep: point planes z0..z1 as bit masks, computed from the
        // samples (the masks of plane k+1 are loaded while plane k is ranked).
        if constexpr (!EMIT)
            load_plane<T>(vol, g.pts, g.iso, g.iso_u16, x0, y0, z0, S.mask[z0 & 1], lane);
        for (uint32_t k = z0; k <= kend; ++k) {
            const int cur = k & 1, prv = cur ^ 1;
            const int lp = EMIT ? cur : 0;                 // list slot of this plane
            const bool have_plane = k < g.cells.z;
            uint32_t L = 0;
            if constexpr (EMIT) {
                if (have_plane) L = emit_plane<T>(cells, g, vol, tab, out, err, k, z1, xs, yb, cur, lane, S, M);
            } else {
                const uint64_t rowmask = ((1ull << min((uint32_t)ROWS, g.cells.y - y0)) - 1ull);
                load_plane<T>(vol, g.pts, g.iso, g.iso_u16, x0, y0, k + 1, S.mask[(k + 1) & 1], lane);
                __syncwarp();
                const uint64_t *mk = S.mask[cur].lt, *mk1 = S.mask[(k + 1) & 1].lt;
                uint64_t act[GROUPS];
#pragma unroll
                for (int j = 0; j < GROUPS; ++j) {
                    const int c = lane + 32 * j;
                    act[j] = (x0 + c < g.cells.x) ? active_rows(mk[c], mk[c + 1], mk1[c], mk1[c + 1]) & rowmask : 0ull;
                }
                // bit transpose: lane r gets row r's active cells in x order
                uint32_t xr[GROUPS];
                uint32_t cnt = 0;
#pragma unroll
                for (int j = 0; j < GROUPS; ++j) {
                    xr[j] = warp_transpose32((uint32_t)act[j], lane);
                    cnt += __popc(xr[j]);
                }
                const uint32_t inc = warp_incl_scan(cnt, lane);
                L = __shfl_sync(0xffffffffu, inc, 31);
                const uint32_t start = inc - cnt;
                S.rowstart[cur][lane] = (uint16_t)start;
                if (lane == 0) { S.rowstart[cur][32] = (uint16_t)L; S.rowstart[cur][33] = (uint16_t)L; }
                // the slot header for the emit sweep: row starts, and the rows
                // whose first cell (column 0) is active
                const uint32_t col0 = __ballot_sync(0xffffffffu, xr[0] & 1u);
                {
                    uint32_t *h = slot_hdr(cells, g, cell_slot(g, k, yb, xs));
                    const uint32_t lo = __shfl_sync(0xffffffffu, start, (2 * lane) & 31);
                    const uint32_t hi = __shfl_sync(0xffffffffu, start, (2 * lane + 1) & 31);
                    if (lane < 16) h[lane] = lo | (hi << 16);
                    if (lane == 16) { h[16] = L | (L << 16); h[17] = col0; }
                }
                // lane r lists row r in x order
                {
                    uint32_t pos = start;
#pragma unroll
                    for (int j = 0; j < GROUPS; ++j) {
                        uint32_t w = xr[j];
                        while (w) {
                            const int l = __ffs(w) - 1;
                            w &= w - 1;
                            M.set_lst(lp, pos++, (lane << 8) | (32 * j + l));
                        }
                    }
                }
                __syncwarp();
            }
            // count sweep: the ranked active cells, 32 at a time, classified
            // and recorded in the cell store
            if constexpr (!EMIT) {
                uint32_t run = 0;
                uint32_t *const recs = slot_rec(cells, g, cell_slot(g, k, yb, xs));
                const uint64_t *mk = S.mask[cur].lt, *mk1 = S.mask[(k + 1) & 1].lt;
                // can a sample equal the isovalue (uint16: only an integer isovalue)?
                const bool can_eq = std::is_same<T, float>::value || g.isole_u16 == g.iso_u16 + 1u;
                for (uint32_t base = 0; base < L; base += 32) {
                    const uint32_t i = base + lane;
                    const bool valid = i < L;
                    uint32_t packed = 0;
                    int r = 0;
                    if (valid) {
                        const uint32_t e = M.lst(lp, i);
                        r = e >> 8;
                        const int c = e & 0xff;
                        const uint32_t x = x0 + c, y = y0 + r;
                        const uint32_t cfg = cfg_from_masks(mk[c], mk[c + 1], mk1[c], mk1[c + 1], r);
                        Corners4 eqs{0.f, 0.f, 0.f, 0.f};
                        if (can_eq) eqs = load_corners4(vol, g, x, y, k, cfg);
                        const bool l2 = needs_lut2(vol, g, tab, cfg, mk, mk1, c, r, x, y, k);
                        uint32_t le4 = le4_from_masks(mk[c + 1], mk1[c], mk1[c + 1], r);   // below
                        if (can_eq) le4 |= corner_eq4(eqs, g.iso);                           // or at
                        const uint32_t info = info_from_bits(cfg, le4);
                        recs[i] = rec_pack((uint32_t)c, (uint32_t)r, cfg, l2, info);
                        n_l2 += l2;
                        packed = (nvert_of(tab, cfg, l2) + __popc(info & 7u)) |
                                 (quad_count(info, cfg, x, y, k, g.cells, n_drop) << 16);
                    }
                    const uint32_t incl = warp_incl_scan(packed, lane);
                    const uint32_t ex = run + incl - packed;
                    run += __shfl_sync(0xffffffffu, incl, 31);
                    if (valid && i == S.rowstart[cur][r]) S.rowbase[r] = ex;
                    __syncwarp();
                    if (valid && i + 1 == S.rowstart[cur][r + 1]) S.rowtot[r] = ex + packed - S.rowbase[r];
                    __syncwarp();
                }
                if (y0 + lane < g.cells.y) {
                    const uint32_t t = S.rowstart[cur][lane] == S.rowstart[cur][lane + 1] ? 0u : S.rowtot[lane];
                    seg_cnt[seg_index(g, k, y0 + lane, xs)] = t;   // vertices | quads << 16
                }
                n_act += L;
            }
            // quads of own cells of plane k-1: their +z ring cells are in plane
            // k.  The plane's quads were listed in order as its cells were
            // classified; each lane writes one.
            if constexpr (EMIT) if (k > z0) {
                const uint32_t Qp = S.qn[prv];
                for (uint32_t t = lane; t < Qp; t += 32) {
                    const uint32_t item = M.qitem(prv, t);
                    const uint32_t i = item & 0x1fffu;
                    const int s = (int)(item >> 13);
                    const uint32_t e = M.lst(prv, i);
                    const int r = e >> 8, c = e & 0xff;
                    const uint32_t info = M.info(prv, i);   // wanted edges (bits 0-2), ccw bits (3-5)
                    const uint64_t q = (uint64_t)S.segq[prv][r] + cell_qrel(M.ent(prv, i)) +
                                       __popc(info & 7u & ((1u << s) - 1u));
                    if (q >= out.qcap) {
                        atomicOr(err, DEV_ERR_OVERFLOW);
                        continue;
                    }
                    // The ring cells of the quad, by list index: the owner (c, r)
                    // of plane k-1 and the first cells at or after column c of
                    // row r+1 of plane k-1 (r1), and of rows r (r2) and r+1 (r3)
                    // of plane k, each possibly followed by its +x neighbour, the
                    // next entry of its row.
                    const uint32_t qc = (uint32_t)c >> 5, bm = (1u << (c & 31)) - 1u;
                    const uint32_t m0 = qc > 0 ? ~0u : bm, m1 = qc > 1 ? ~0u : (qc == 1 ? bm : 0u);
                    const uint32_t m2 = qc > 2 ? ~0u : (qc == 2 ? bm : 0u), m3 = qc == 3 ? bm : 0u;
                    auto rank = [&](int pl, int rr) -> uint32_t {
                        const uint4 w = *reinterpret_cast<const uint4 *>(S.xrow[pl][rr]);
                        return S.rowstart[pl][rr] + __popc(w.x & m0) + __popc(w.y & m1) + __popc(w.z & m2) +
                               __popc(w.w & m3);
                    };
                    const uint32_t ox = i | (rank(prv, r + 1) << 16), oy = rank(cur, r) | (rank(cur, r + 1) << 16);
                    const uint32_t ring = s == 0 ? kRing6 : (s == 1 ? kRing9 : kRing10);
                    const bool ccw = (info >> (s + 3)) & 1u;
                    uint32_t idx[4];
                    bool bad = false;
#pragma unroll
                    for (int it = 0; it < 4; ++it) {
                        const int kk = ccw ? it : (4 - it) & 3;    // ccw 0,1,2,3; cw 0,3,2,1 (dmc.cu:1636-1645)
                        const uint32_t sl = (ring >> (8 * kk)) & 0xffu;
                        const int pl = (sl & 1u) ? cur : prv;
                        const uint32_t plus = (sl >> 3) & 1u, rr = (uint32_t)r + ((sl >> 4) & 1u);
                        // base entry (sl bits 1-2): owner, r1, r2, r3; then its +x neighbour
                        const uint32_t bsel = (sl >> 1) & 3u;
                        const uint32_t bw = bsel < 2 ? ox : oy;
                        const uint32_t li = ((bsel & 1u) ? (bw >> 16) : (bw & 0xffffu)) + plus;
                        const bool ok = li < S.rowstart[pl][HROWS];
                        const uint32_t rd = ok ? M.ent(pl, li) : 0u;
                        const uint32_t m = lut_m(tab, cell_cfg(rd), cell_l2(rd), (int)ring_edge(s, kk));
                        bad |= !ok || m == 0xffu;
                        idx[it] = S.segv[pl][rr][(c + (int)plus) == W ? 1 : 0] + cell_vrel(rd) + (m == 0xffu ? 0u : m) - g.vbase;
                    }
                    if (bad) atomicOr(err, DEV_ERR_BOUNDS);
                    reinterpret_cast<uint4 *>(out.quads)[q] = make_uint4(idx[0], idx[1], idx[2], idx[3]);
                    if (out.tris) {
                        uint32_t *tp = out.tris + 6 * q;   // 4-byte stores: callers' buffers need only 4-byte alignment
                        tp[0] = idx[0]; tp[1] = idx[1]; tp[2] = idx[2];
                        tp[3] = idx[2]; tp[4] = idx[3]; tp[5] = idx[0];
                    }
                }
            }
            __syncwarp();
        }
    }
    if constexpr (!EMIT) if (!(range.flags & kNoStats)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            n_l2 += __shfl_xor_sync(0xffffffffu, n_l2, o);
            n_drop += __shfl_xor_sync(0xffffffffu, n_drop, o);
        }
        if (lane == 0) {
            if (n_act) atomicAdd(&counters[0], (unsigned long long)n_act);
            if (n_l2) atomicAdd(&counters[1], (unsigned long long)n_l2);
            if (n_drop) atomicAdd(&counters[2], (unsigned long long)n_drop);
        }
    }
}

// Start of a pipeline launch: zero the scan tiles, tickets and control block
// and fill each volume's point coordinates x(i) = ijk_to_xyz(i, cells.x, ...)
// (utils.hpp:118-122).  Blocks stride over volumes, threads over points.
__global__ void batch_prep(const BatchHead *__restrict__ head, TileState *tiles, uint32_t *tickets, DevCtl *ctl)
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (uint32_t t = tid; t < head->n_tiles; t += nth) tiles[t] = TileState{};
    if (tid < kTickets) tickets[tid] = 0;
    if (tid < sizeof(DevCtl) / 4) reinterpret_cast<uint32_t *>(ctl)[tid] = 0;
    const Geom *vols = batch_geoms(head);
    for (uint32_t v = blockIdx.x; v < head->n; v += gridDim.x) {
        const Geom &g = vols[v];
        float *coord = const_cast<float *>(g.coord);
        const uint32_t n = g.pts.x + g.pts.y + g.pts.z;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            float c;
            if (i < g.pts.x) c = ijk_to_xyz(i, g.cells.x, g.rng.x, g.mn.x);
            else if (i < g.pts.x + g.pts.y) c = ijk_to_xyz(i - g.pts.x, g.cells.y, g.rng.y, g.mn.y);
            else c = ijk_to_xyz(i - g.pts.x - g.pts.y, g.cells.z, g.rng.z, g.mn.z);
            coord[i] = c;
        }
    }
}

// After the scan: each volume's first vertex / quad and its counts.
__global__ void volume_results(BatchHead *head, const uint32_t *seg_cnt, const uint2 *seg_off,
                               const unsigned long long *totals, dmc_batch_result *res)
{
    Geom *vols = const_cast<Geom *>(batch_geoms(head));
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < head->n; v += gridDim.x * blockDim.x) {
        Geom &g = vols[v];
        dmc_batch_result r{0, 0, 0, 0};
        if (!g.nseg) {
            // no cells: an empty slice where the next volume starts
            if (g.seg_base < head->nseg) { r.vertex_offset = seg_off[g.seg_base].x; r.quad_offset = seg_off[g.seg_base].y; }
            else { r.vertex_offset = totals[0]; r.quad_offset = totals[1]; }
        } else {
            const uint2 f = seg_off[g.seg_base], lo = seg_off[g.seg_base + g.nseg - 1];
            const uint32_t lc = seg_cnt[g.seg_base + g.nseg - 1];
            r.vertex_offset = f.x; r.n_vertices = (unsigned long long)lo.x + (lc & 0xffffu) - f.x;
            r.quad_offset = f.y; r.n_quads = (unsigned long long)lo.y + (lc >> 16) - f.y;
            g.vbase = f.x; g.qbase = f.y;
        }
        if (res) res[g.item] = r;
    }
}

// Running totals and error word after a slab's scan, written to mapped host
// memory so that the host learns each slab's output range while later slabs
// are still uploading.
__global__ void snap_totals(const DevCtl *ctl, unsigned long long *dst)
{
    if (threadIdx.x == 0) {
        dst[0] = ctl->totals[0];
        dst[1] = ctl->totals[1];
        dst[2] = ctl->err;
    }
}

// ---------------------------------------------------------------------------
// segment scan (decoupled look-back)

// Scans segments [seg_lo, seg_lo + seg_cnt) (clipped to the plan's segments).
__global__ void __launch_bounds__(SCAN_NT) seg_scan(const BatchHead *__restrict__ head, const uint32_t *__restrict__ cnt,
                                                    ScanCtl ctl, uint2 *__restrict__ off, uint64_t seg_lo, uint64_t seg_cnt)
{
    __shared__ uint32_t s_slot;
    __shared__ unsigned long long s_warp[SCAN_NT / 32 + 1];
    __shared__ unsigned long long s_ex[2];
    const uint64_t rest = seg_lo >= head->nseg ? 0ull : (uint64_t)head->nseg - seg_lo;
    const uint64_t n = rest < seg_cnt ? rest : seg_cnt;
    cnt += seg_lo;
    off += seg_lo;
    ctl.n_tiles = (uint32_t)((n + SCAN_TILE - 1) / SCAN_TILE);
    // tiles are claimed in order, so a tile only waits on tiles whose blocks already run
    for (;;) {
        const uint32_t tile = claim_tile(ctl.ticket, &s_slot);
        if (tile >= ctl.n_tiles) break;
        const uint64_t first = (uint64_t)tile * SCAN_TILE + (uint64_t)threadIdx.x * SCAN_ITEMS;
        // a segment's count is vertices | quads << 16 (at most 7 and 3 per
        // cell of a 128-cell row), so the packed words of a thread's items
        // add without a carry between the halves
        uint32_t c[SCAN_ITEMS];
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            c[i] = first + i < n ? cnt[first + i] : 0u;
            sum += c[i];
        }
        const uint32_t sv = sum & 0xffffu, sq = sum >> 16;
        unsigned long long tot;
        unsigned long long ex = block_exclusive_scan<SCAN_NT>((unsigned long long)sv | ((unsigned long long)sq << 32), s_warp, &tot);
        tile_prefix(ctl, tile, (uint32_t)tot, (uint32_t)(tot >> 32), s_ex);
        unsigned long long bv = s_ex[0] + (uint32_t)ex, bq = s_ex[1] + (uint32_t)(ex >> 32);
#pragma unroll
        for (int i = 0; i < SCAN_ITEMS; ++i) {
            if (first + i < n) off[first + i] = make_uint2((uint32_t)bv, (uint32_t)bq);
            bv += c[i] & 0xffffu; bq += c[i] >> 16;
        }
    }
}

}  // namespace brick

// ---------------------------------------------------------------------------
// host side

bool brick_supports(const ExtractArgs &a)
{
    return a.cells.x >= 1 && a.cells.y >= 1 && a.cells.z >= 1;
}

constexpr size_t kEmitSmem = brick::kTablesBytes + sizeof(brick::EmitSmem) * brick::NWB_EMIT;
constexpr size_t kCountSmem = brick::kTablesBytes + sizeof(brick::CountSmem) * brick::NWB_COUNT;
// three emit blocks and three count blocks per SM (228 KB of shared memory,
// 1 KB of it reserved per block); what is left of the 256 KB is L1, which the
// emit sweep's corner gathers use
static_assert(3 * (kEmitSmem + 1024) <= 228 * 1024, "emit sweep: three blocks per SM must fit");
static_assert(3 * (kCountSmem + 1024) <= 228 * 1024, "count sweep: three blocks per SM must fit");

template <class T, bool EMIT>
static int sweep_grid(Ctx *ctx)
{
    using namespace brick;
    const size_t smem = EMIT ? kEmitSmem : kCountSmem;
    cudaFuncSetAttribute(brick_sweep<T, EMIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int b = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, brick_sweep<T, EMIT>, 32 * nwb(EMIT), smem);
    if (b < 1) b = 1;
    return b * ctx->num_sms;
}

static void iso_thresholds(float f, uint32_t &lt, uint32_t &le)
{
    // uint16 samples: v < iso <=> v < lt;  v <= iso <=> v < le (floor(iso) + 1)
    if (!(f > 0.f)) lt = 0;                       // also NaN
    else if (f > 65535.f) lt = 65536;
    else { const uint32_t fl = (uint32_t)f; lt = ((float)fl == f) ? fl : fl + 1; }
    if (!(f >= 0.f)) le = 0;
    else if (f >= 65535.f) le = 65536;
    else le = (uint32_t)f + 1;
}

// Cell store of one volume: a header and a record area per slot (cell plane
// of a brick), 4 bytes per cell of its bricks plus 80 bytes per slot.
static uint64_t cell_words(const BrickItem &it)
{
    using namespace brick;
    if (it.cells.x == 0 || it.cells.y == 0 || it.cells.z == 0) return 0;
    const uint64_t nslots = (uint64_t)it.cells.z * ((it.cells.y + ROWS - 1) / ROWS) * ((it.cells.x + W - 1) / W);
    return nslots * (kHdrWords + kRecWords);
}

// Per-context pipeline state.  Scratch (device) and staging (pinned host) are
// laid out for capacities that only grow; a captured graph holds the
// addresses of both, plus the output buffers, and is re-captured when any of
// them changes.
struct BatchState {
    // capacities of the layout
    uint32_t cap_items = 0;
    uint64_t cap_seg = 0, cap_coord = 0, cap_cell = 0;
    uint64_t layout_gen = 0;           // scratch_gen the layout was carved for (0: none)
    uint64_t layout_id = 0;            // bumped on every re-carve: captured graphs hold the addresses
    // device layout (inside ctx->scratch)
    brick::BatchHead *d_plan = nullptr;
    uint32_t *seg_cnt = nullptr;   // per segment: vertices | quads << 16
    uint2 *seg_off = nullptr;
    TileState *tiles = nullptr;
    brick::Spill *spill = nullptr;
    uint32_t *cells = nullptr;          // cell store, cap_cell words
    float *coord = nullptr;
    dmc_batch_result *d_res = nullptr;
    uint32_t *tickets = nullptr;
    size_t plan_bytes = 0;
    // pinned staging: plan, then the per-volume results
    void *h_stage = nullptr;
    size_t h_stage_bytes = 0;
    uint64_t stage_gen = 0;
    // grids of the persistent sweeps [dtype][emit]
    int grid[2][2] = {{0, 0}, {0, 0}};
    // cached graph, the layout it was captured for, and its emit nodes,
    // whose output arguments are rewritten when a batch targets other buffers
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    uint64_t g_layout_id = 0, g_stage_gen = 0;
    cudaGraphNode_t emit_node[2] = {nullptr, nullptr};
    cudaKernelNodeParams emit_params[2]{};
    brick::EmitOut g_out{};
    // the count sweeps and the scan, whose grids are resized to each batch
    cudaGraphNode_t count_node[2] = {nullptr, nullptr}, scan_node = nullptr;
    cudaKernelNodeParams count_params[2]{}, scan_params{};
    int g_grid[2][2] = {{0, 0}, {0, 0}}, g_scan_grid = 0;   // grids the instantiated graph runs now
    // streamed host extraction: copy streams, per-slab events and mapped
    // snapshots of the running totals (vertices, quads, error word per slab)
    cudaStream_t s_in = nullptr, s_out = nullptr;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_in[brick::kMaxSlabs]{}, ev_tot[brick::kMaxSlabs]{}, ev_emit[brick::kMaxSlabs]{};
    unsigned long long *h_snap = nullptr, *d_snap = nullptr;
    // sharded extraction between its two phases: sample type, z-brick range, bricks per z layer
    bool shard_ready = false;
    uint64_t sh_scratch_gen = 0;       // the scratch the count phase left its plan and offsets in
    int sh_grp = 0;
    uint32_t sh_zb0 = 0, sh_zb1 = 0;
    uint64_t sh_bxy = 0;
    // batch in flight
    bool in_flight = false;
    uint32_t n_inflight = 0;
    cudaEvent_t done = nullptr;
};

// Resident warps of the largest sweep launch: one spill slot each, and the
// unit of the planes-per-brick rule.
static uint64_t sweep_warps(const BatchState &b)
{
    using namespace brick;
    uint64_t w = 0;
    for (int t = 0; t < 2; ++t)
        w = std::max<uint64_t>(w, std::max<uint64_t>((uint64_t)b.grid[t][0] * NWB_COUNT, (uint64_t)b.grid[t][1] * NWB_EMIT));
    return w;
}

void batch_state_free(Ctx *ctx)
{
    BatchState *b = ctx->batch;
    if (!b) return;
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->done) cudaEventDestroy(b->done);
    if (b->h_stage) cudaFreeHost(b->h_stage);
    if (b->s_in) cudaStreamDestroy(b->s_in);
    if (b->s_out) cudaStreamDestroy(b->s_out);
    if (b->ev_start) cudaEventDestroy(b->ev_start);
    for (int i = 0; i < brick::kMaxSlabs; ++i) {
        if (b->ev_in[i]) cudaEventDestroy(b->ev_in[i]);
        if (b->ev_tot[i]) cudaEventDestroy(b->ev_tot[i]);
        if (b->ev_emit[i]) cudaEventDestroy(b->ev_emit[i]);
    }
    if (b->h_snap) cudaFreeHost(b->h_snap);
    delete b;
    ctx->batch = nullptr;
}

static dmc_status batch_state(Ctx *ctx, BatchState **out)
{
    if (!ctx->batch) {
        BatchState *b = new (std::nothrow) BatchState();
        if (!b) return DMC_ERR_OOM;
        ctx->batch = b;
        b->grid[0][0] = sweep_grid<float, false>(ctx);
        b->grid[0][1] = sweep_grid<float, true>(ctx);
        b->grid[1][0] = sweep_grid<uint16_t, false>(ctx);
        b->grid[1][1] = sweep_grid<uint16_t, true>(ctx);
        CUDA_TRY(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
    }
    *out = ctx->batch;
    return DMC_OK;
}

// Carves the scratch and staging for at least the given capacities.
static dmc_status batch_layout(Ctx *ctx, BatchState &b, uint32_t items, uint64_t seg, uint64_t ncoord, uint64_t ncell)
{
    using namespace brick;
    const bool fits = b.layout_gen == ctx->scratch_gen && items <= b.cap_items && seg <= b.cap_seg &&
                      ncoord <= b.cap_coord && ncell <= b.cap_cell;
    if (fits) return DMC_OK;
    // grow with headroom so that a stream of similar batches settles on one layout
    b.cap_items = std::max<uint32_t>(b.cap_items, items + items / 4 + 1);
    b.cap_seg = std::max<uint64_t>(b.cap_seg, seg + seg / 4 + SCAN_TILE);
    b.cap_coord = std::max<uint64_t>(b.cap_coord, ncoord + ncoord / 4 + 64);
    b.cap_cell = std::max<uint64_t>(b.cap_cell, ncell + ncell / 4 + 64);
    const uint64_t cap_tiles = (b.cap_seg + SCAN_TILE - 1) / SCAN_TILE;
    b.plan_bytes = sizeof(BatchHead) + sizeof(Geom) * (size_t)b.cap_items;
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t r = off; off += (bytes + 255) & ~(size_t)255; return r; };
    const size_t o_plan = carve(b.plan_bytes);
    const size_t o_cnt = carve(4 * b.cap_seg), o_off = carve(8 * b.cap_seg);
    const size_t o_tiles = carve(sizeof(TileState) * (cap_tiles + kMaxSlabs));   // slabs: one partial tile each
    const size_t o_spill = carve(sizeof(Spill) * (size_t)sweep_warps(b));
    const size_t o_cell = carve(4 * b.cap_cell);
    const size_t o_coord = carve(4 * b.cap_coord);
    const size_t o_res = carve(sizeof(dmc_batch_result) * (size_t)b.cap_items);
    const size_t o_tk = carve(4 * kTickets);
    if (b.in_flight) return DMC_ERR_INVALID_ARG;
    dmc_status s = ctx_reserve_scratch(ctx, off);
    if (s != DMC_OK) return s;
    uint8_t *base = (uint8_t *)ctx->scratch;
    b.d_plan = (BatchHead *)(base + o_plan);
    b.seg_cnt = (uint32_t *)(base + o_cnt);
    b.seg_off = (uint2 *)(base + o_off);
    b.tiles = (TileState *)(base + o_tiles);
    b.spill = (Spill *)(base + o_spill);
    b.cells = (uint32_t *)(base + o_cell);
    b.coord = (float *)(base + o_coord);
    b.d_res = (dmc_batch_result *)(base + o_res);
    b.tickets = (uint32_t *)(base + o_tk);
    b.layout_gen = ctx->scratch_gen;
    ++b.layout_id;
    const size_t stage = b.plan_bytes + sizeof(dmc_batch_result) * (size_t)b.cap_items;
    if (stage > b.h_stage_bytes) {
        if (b.h_stage) { CUDA_TRY(cudaDeviceSynchronize()); cudaFreeHost(b.h_stage); b.h_stage = nullptr; b.h_stage_bytes = 0; }
        CUDA_TRY(cudaMallocHost(&b.h_stage, stage));
        b.h_stage_bytes = stage;
        ++b.stage_gen;
    }
    return DMC_OK;
}

static dmc_batch_result *stage_results(BatchState &b)
{
    return (dmc_batch_result *)((uint8_t *)b.h_stage + b.plan_bytes);
}

// Blocks of a sweep launch: the resident grid, or fewer when the launch has
// fewer bricks than resident warps, so that small extractions do not start
// (and stage tables in) hundreds of idle blocks.  A captured graph keeps the
// full grid: it replays batches of any size.
static int sweep_blocks(const BatchState &b, int t, bool emit, uint64_t nbricks, bool full_grid)
{
    using namespace brick;
    const int full = b.grid[t][emit ? 1 : 0];
    if (full_grid) return full;
    const uint64_t nwb = emit ? NWB_EMIT : NWB_COUNT;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)full, (nbricks + nwb - 1) / nwb));
}

// Front half: plan upload, prep, count sweeps, scan, per-volume offsets.
// Sweeps of a sample type without bricks are skipped unless `all` (a graph
// must serve any later mix of types).
static dmc_status enqueue_front(Ctx *ctx, BatchState &b, dmc_batch_result *d_res, bool timed, const uint64_t nb[2],
                                bool all, cudaStream_t st)
{
    NvtxRange nvtx("dmc count sweep and scan (enqueue)");
    using namespace brick;
    CUDA_TRY(cudaMemcpyAsync(b.d_plan, b.h_stage, b.plan_bytes, cudaMemcpyHostToDevice, st));
    batch_prep<<<2 * ctx->num_sms, 256, 0, st>>>(b.d_plan, b.tiles, b.tickets, ctx->d_ctl);
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecord(ctx->evk[0], st));
    if (all || nb[0]) {
        brick_sweep<float, false><<<sweep_blocks(b, 0, false, nb[0], all), 32 * NWB_COUNT, kCountSmem, st>>>(
            b.d_plan, 0, BrickRange{0, kAllBricks}, ctx->d_tab, b.seg_cnt, EmitOut{}, b.spill, b.cells, &b.tickets[0], ctx->d_ctl->counters, &ctx->d_ctl->err);
        CUDA_TRY(cudaGetLastError());
    }
    if (all || nb[1]) {
        brick_sweep<uint16_t, false><<<sweep_blocks(b, 1, false, nb[1], all), 32 * NWB_COUNT, kCountSmem, st>>>(
            b.d_plan, 1, BrickRange{0, kAllBricks}, ctx->d_tab, b.seg_cnt, EmitOut{}, b.spill, b.cells, &b.tickets[1], ctx->d_ctl->counters, &ctx->d_ctl->err);
        CUDA_TRY(cudaGetLastError());
    }
    if (timed) CUDA_TRY(cudaEventRecord(ctx->evk[1], st));
    ScanCtl ctl;
    ctl.tiles = b.tiles; ctl.ticket = &ctx->d_ctl->ticket; ctl.err = &ctx->d_ctl->err;
    ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = 0;
    const uint32_t n_tiles = ((const BatchHead *)b.h_stage)->n_tiles;
    const int scan_blocks = all ? 2 * ctx->num_sms : (int)std::max<uint32_t>(1u, std::min<uint32_t>(2u * ctx->num_sms, n_tiles));
    seg_scan<<<scan_blocks, SCAN_NT, 0, st>>>(b.d_plan, b.seg_cnt, ctl, b.seg_off, 0ull, ~0ull);
    CUDA_TRY(cudaGetLastError());
    volume_results<<<4, 128, 0, st>>>(b.d_plan, b.seg_cnt, b.seg_off, ctx->d_ctl->totals, d_res);
    CUDA_TRY(cudaGetLastError());
    if (timed) CUDA_TRY(cudaEventRecord(ctx->evk[2], st));
    return DMC_OK;
}

// Back half: emit sweeps, then the control block and results to pinned memory.
static dmc_status enqueue_back(Ctx *ctx, BatchState &b, const brick::EmitOut &eo, dmc_batch_result *d_res, bool timed,
                               const uint64_t nb[2], bool all, cudaStream_t st)
{
    NvtxRange nvtx("dmc emit sweep (enqueue)");
    using namespace brick;
    if (timed) CUDA_TRY(cudaEventRecord(ctx->evk[3], st));
    if (all || nb[0]) {
        brick_sweep<float, true><<<sweep_blocks(b, 0, true, nb[0], all), 32 * NWB_EMIT, kEmitSmem, st>>>(
            b.d_plan, 0, BrickRange{0, kAllBricks}, ctx->d_tab, nullptr, eo, b.spill, b.cells, &b.tickets[2], ctx->d_ctl->counters, &ctx->d_ctl->err);
        CUDA_TRY(cudaGetLastError());
    }
    if (all || nb[1]) {
        brick_sweep<uint16_t, true><<<sweep_blocks(b, 1, true, nb[1], all), 32 * NWB_EMIT, kEmitSmem, st>>>(
            b.d_plan, 1, BrickRange{0, kAllBricks}, ctx->d_tab, nullptr, eo, b.spill, b.cells, &b.tickets[3], ctx->d_ctl->counters, &ctx->d_ctl->err);
        CUDA_TRY(cudaGetLastError());
    }
    if (timed) CUDA_TRY(cudaEventRecord(ctx->evk[4], st));
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(stage_results(b), d_res, sizeof(dmc_batch_result) * (size_t)b.cap_items,
                             cudaMemcpyDeviceToHost, st));
    return DMC_OK;
}

static void stats_from_ctl(Ctx *ctx)
{
    ctx->stats.n_vertices = ctx->h_ctl->totals[0];
    ctx->stats.n_quads = ctx->h_ctl->totals[1];
    ctx->stats.n_active_cells = ctx->h_ctl->counters[0];
    ctx->stats.n_lut2_cells = ctx->h_ctl->counters[1];
    ctx->stats.n_dropped_quads = ctx->h_ctl->counters[2];
}

static dmc_status ctl_status(const DevCtl *c)
{
    if (c->err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    if (c->err & DEV_ERR_OVERFLOW) return DMC_ERR_OUTPUT_OVERFLOW;
    if (c->err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    if (c->totals[0] >= 0xFFFFFFFFull || c->totals[1] >= 0xFFFFFFFFull) return DMC_ERR_OUTPUT_OVERFLOW;
    return DMC_OK;
}

static bool same_out(const brick::EmitOut &a, const brick::EmitOut &b)
{
    return a.seg_off == b.seg_off && a.verts == b.verts && a.vcap == b.vcap && a.quads == b.quads &&
           a.qcap == b.qcap && a.tris == b.tris;
}

// Captures the whole pipeline (both sample types) on the context's own
// stream; the graph is later launched on the caller's stream.
static dmc_status capture_graph(Ctx *ctx, BatchState &b, const brick::EmitOut &eo, const uint64_t nb[2])
{
    using namespace brick;
    if (b.gexec) { cudaGraphExecDestroy(b.gexec); b.gexec = nullptr; }
    if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
    b.emit_node[0] = b.emit_node[1] = nullptr;
    b.count_node[0] = b.count_node[1] = nullptr;
    b.scan_node = nullptr;
    cudaGraph_t graph = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    dmc_status cs = enqueue_front(ctx, b, b.d_res, false, nb, true, ctx->stream);
    if (cs == DMC_OK) cs = enqueue_back(ctx, b, eo, b.d_res, false, nb, true, ctx->stream);
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
    if (cs != DMC_OK) { if (graph) cudaGraphDestroy(graph); return cs; }
    CUDA_TRY(ce);
    // the sweep and scan nodes, found by kernel
    size_t nn = 0;
    CUDA_TRY(cudaGraphGetNodes(graph, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CUDA_TRY(cudaGraphGetNodes(graph, nodes.data(), &nn));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType t;
        CUDA_TRY(cudaGraphNodeGetType(nd, &t));
        if (t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        CUDA_TRY(cudaGraphKernelNodeGetParams(nd, &kp));
        for (int g = 0; g < 2; ++g) {
            const void *fe = g ? (const void *)brick_sweep<uint16_t, true> : (const void *)brick_sweep<float, true>;
            const void *fc = g ? (const void *)brick_sweep<uint16_t, false> : (const void *)brick_sweep<float, false>;
            if (kp.func == fe) { b.emit_node[g] = nd; b.emit_params[g] = kp; }
            if (kp.func == fc) { b.count_node[g] = nd; b.count_params[g] = kp; }
        }
        if (kp.func == (const void *)seg_scan) { b.scan_node = nd; b.scan_params = kp; }
    }
    if (!b.emit_node[0] || !b.emit_node[1] || !b.count_node[0] || !b.count_node[1] || !b.scan_node) {
        cudaGraphDestroy(graph);
        return DMC_ERR_CUDA;
    }
    for (int g = 0; g < 2; ++g) {
        b.g_grid[g][0] = (int)b.count_params[g].gridDim.x;
        b.g_grid[g][1] = (int)b.emit_params[g].gridDim.x;
    }
    b.g_scan_grid = (int)b.scan_params.gridDim.x;
    ce = cudaGraphInstantiate(&b.gexec, graph, 0);
    if (ce != cudaSuccess) { cudaGraphDestroy(graph); CUDA_TRY(ce); }
    b.graph = graph;
    b.g_layout_id = b.layout_id;
    b.g_stage_gen = b.stage_gen;
    b.g_out = eo;
    return DMC_OK;
}

// Points the graph's emit sweeps at other output buffers (same arguments as
// the launches in enqueue_back, with a new EmitOut) and sizes the sweep and
// scan grids to this batch's bricks and tiles (a small batch then starts no
// idle persistent blocks).  Nodes are rewritten only when something changed.
static dmc_status retarget_graph(Ctx *ctx, BatchState &b, const brick::EmitOut &eo, const uint64_t nb[2])
{
    using namespace brick;
    const uint32_t n_tiles = ((const BatchHead *)b.h_stage)->n_tiles;
    const int scan_grid = (int)std::max<uint32_t>(1u, std::min<uint32_t>(2u * ctx->num_sms, n_tiles));
    if (scan_grid != b.g_scan_grid) {
        cudaKernelNodeParams kp = b.scan_params;
        kp.gridDim = dim3((unsigned)scan_grid);
        CUDA_TRY(cudaGraphExecKernelNodeSetParams(b.gexec, b.scan_node, &kp));
        b.g_scan_grid = scan_grid;
    }
    bool emit_grid_changed = false;
    int want[2][2];
    for (int g = 0; g < 2; ++g) {
        want[g][0] = sweep_blocks(b, g, false, nb[g], false);
        want[g][1] = sweep_blocks(b, g, true, nb[g], false);
        if (want[g][0] != b.g_grid[g][0]) {
            cudaKernelNodeParams kp = b.count_params[g];
            kp.gridDim = dim3((unsigned)want[g][0]);
            CUDA_TRY(cudaGraphExecKernelNodeSetParams(b.gexec, b.count_node[g], &kp));
            b.g_grid[g][0] = want[g][0];
        }
        emit_grid_changed |= want[g][1] != b.g_grid[g][1];
    }
    if (same_out(eo, b.g_out) && !emit_grid_changed) return DMC_OK;
    for (uint32_t g = 0; g < 2; ++g) {
        const BatchHead *a_head = b.d_plan;
        uint32_t a_group = g;
        BrickRange a_range{0, kAllBricks};
        const DeviceTables *a_tab = ctx->d_tab;
        uint2 *a_cnt = nullptr;
        EmitOut a_out = eo;
        Spill *a_spill = b.spill;
        uint32_t *a_cells = b.cells;
        uint32_t *a_ticket = &b.tickets[2 + g];
        unsigned long long *a_counters = ctx->d_ctl->counters;
        uint32_t *a_err = &ctx->d_ctl->err;
        void *args[] = {&a_head, &a_group, &a_range, &a_tab, &a_cnt, &a_out, &a_spill, &a_cells, &a_ticket, &a_counters, &a_err};
        cudaKernelNodeParams kp = b.emit_params[g];
        kp.kernelParams = args;
        kp.extra = nullptr;
        kp.gridDim = dim3((unsigned)want[g][1]);
        CUDA_TRY(cudaGraphExecKernelNodeSetParams(b.gexec, b.emit_node[g], &kp));
        b.g_grid[g][1] = want[g][1];
    }
    b.g_out = eo;
    return DMC_OK;
}

// Planes per brick: the context's option, or the automatic choice.
static uint32_t pick_zc(Ctx *ctx, const BatchState &b, const BrickItem *items, uint32_t n)
{
    using namespace brick;
    // planes per brick: long sweeps amortise the z halo, but uneven bricks
    // leave warps idle at the end, so keep at least twelve bricks per resident
    // warp (down to two planes per brick; 4 on a 1024^3 volume)
    uint32_t zc = ctx->brick_zc ? ctx->brick_zc : 32;
    if (!ctx->brick_zc) {
        for (;;) {
            uint64_t nb = 0;
            for (uint32_t i = 0; i < n; ++i) {
                const uint3 c = items[i].cells;
                nb += (uint64_t)((c.x + W - 1) / W) * ((c.y + ROWS - 1) / ROWS) * ((c.z + zc - 1) / zc);
            }
            if (zc <= 2 || nb >= 12ull * (uint64_t)sweep_warps(b)) break;
            zc >>= 1;
        }
    }
    return zc;
}

// Chooses the planes per brick and writes the plan (head and one Geom per
// volume: the f32 volumes, then the u16 ones) to the pinned staging, after
// carving the scratch for it.  nb: bricks of each sample type.
static dmc_status stage_plan(Ctx *ctx, BatchState &b, const BrickItem *items, uint32_t n, uint64_t nb[2],
                             uint32_t zc_force = 0)
{
    using namespace brick;
    const uint32_t zc = zc_force ? zc_force : pick_zc(ctx, b, items, n);
    // descriptors: the f32 volumes, then the u16 ones (one launch per type)
    uint64_t nseg = 0, ncoord = 0, ncell = 0;
    nb[0] = nb[1] = 0;
    uint32_t nvol[2] = {0, 0};
    for (uint32_t i = 0; i < n; ++i) {
        const BrickItem &it = items[i];
        nseg += (uint64_t)it.cells.z * it.cells.y * ((it.cells.x + W - 1) / W);
        ncoord += (uint64_t)it.pts.x + it.pts.y + it.pts.z;
        ncell += cell_words(it);
        nvol[it.dtype == DMC_F32 ? 0 : 1]++;
    }
    const uint64_t n_tiles = (nseg + SCAN_TILE - 1) / SCAN_TILE;
    if (n_tiles >= (1ull << 31)) return DMC_ERR_UNSUPPORTED;
    dmc_status s = batch_layout(ctx, b, n, nseg, ncoord, ncell);
    if (s != DMC_OK) return s;
    BatchHead *head = (BatchHead *)b.h_stage;
    Geom *geoms = (Geom *)(head + 1);
    uint32_t pos[2] = {0, nvol[0]};
    uint64_t seg_base = 0, coord_base = 0, cell_base = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const BrickItem &it = items[i];
        const int grp = it.dtype == DMC_F32 ? 0 : 1;
        Geom &g = geoms[pos[grp]++];
        g = Geom{};
        g.data = it.data; g.pts = it.pts; g.cells = it.cells; g.iso = it.iso; g.mn = it.mn; g.rng = it.rng;
        iso_thresholds(it.iso, g.iso_u16, g.isole_u16);
        g.nxs = (it.cells.x + W - 1) / W;
        g.nyb = (it.cells.y + ROWS - 1) / ROWS;
        g.zc = zc;
        g.nzb = (it.cells.z + zc - 1) / zc;
        g.brick_base = nb[grp];
        nb[grp] += (uint64_t)g.nxs * g.nyb * g.nzb;
        g.seg_base = seg_base;
        g.nseg = (uint64_t)it.cells.z * it.cells.y * g.nxs;
        seg_base += g.nseg;
        g.coord = b.coord + coord_base;
        g.cell_base = cell_base;
        cell_base += cell_words(it);
        coord_base += (uint64_t)it.pts.x + it.pts.y + it.pts.z;
        g.item = i;
    }
    if (nb[0] >= 0xF0000000ull || nb[1] >= 0xF0000000ull) return DMC_ERR_UNSUPPORTED;
    head->nbricks[0] = nb[0]; head->nbricks[1] = nb[1];
    head->nseg = nseg;
    head->nvol[0] = nvol[0]; head->nvol[1] = nvol[1];
    head->n = n;
    head->n_tiles = (uint32_t)n_tiles;
    return DMC_OK;
}

// Extraction of one or many volumes: count sweep, one segment scan over all
// volumes, per-volume offsets, emit sweep.  Vertices and quads of volume v
// land at its offsets in the shared output buffers; quad indices are relative
// to the volume's first vertex.
dmc_status brick_extract(Ctx *ctx, const BrickItem *items, uint32_t n, const BrickOut &o, cudaStream_t st)
{
    using namespace brick;
    if (n == 0) return DMC_ERR_INVALID_ARG;
    BatchState *bp = nullptr;
    dmc_status s = batch_state(ctx, &bp);
    if (s != DMC_OK) return s;
    BatchState &b = *bp;
    if (b.in_flight) return DMC_ERR_INVALID_ARG;
    b.shard_ready = false;          // this call replaces a sharded count's plan
    uint64_t nb[2] = {0, 0};
    if ((s = stage_plan(ctx, b, items, n, nb)) != DMC_OK) return s;

    EmitOut eo;
    eo.seg_off = b.seg_off; eo.verts = o.verts; eo.vcap = o.vcap; eo.quads = o.quads; eo.qcap = o.qcap; eo.tris = o.tris;
    dmc_batch_result *d_res = (o.d_results && o.mode != BATCH_GRAPH) ? o.d_results : b.d_res;
    if (o.mode == BATCH_GRAPH) {
        // the graph's per-volume results always go to scratch; a caller's
        // device results are copied from there after the launch
        if (!b.gexec || b.g_layout_id != b.layout_id || b.g_stage_gen != b.stage_gen) {
            if ((s = capture_graph(ctx, b, eo, nb)) != DMC_OK) return s;
        }
        if ((s = retarget_graph(ctx, b, eo, nb)) != DMC_OK) return s;
        CUDA_TRY(cudaGraphLaunch(b.gexec, st));
        if (o.d_results)
            CUDA_TRY(cudaMemcpyAsync(o.d_results, b.d_res, sizeof(dmc_batch_result) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    } else if (o.mode == BATCH_ASYNC) {
        if ((s = enqueue_front(ctx, b, d_res, false, nb, false, st)) != DMC_OK) return s;
        if ((s = enqueue_back(ctx, b, eo, d_res, false, nb, false, st)) != DMC_OK) return s;
    } else {
        if ((s = enqueue_front(ctx, b, d_res, true, nb, false, st)) != DMC_OK) return s;
        ctx->evk_used = 1;
        if (!o.sizing_only) {
            // The emit sweep follows at once: it checks every write against the
            // capacities on the device, so no host round trip sits between the
            // sweeps.  Too small buffers give DMC_ERR_OUTPUT_OVERFLOW with the
            // totals (their contents are then undefined).
            if ((s = enqueue_back(ctx, b, eo, d_res, true, nb, false, st)) != DMC_OK) return s;
            ctx->evk_used = 2;
            CUDA_TRY(cudaStreamSynchronize(st));
            stats_from_ctl(ctx);
            if (o.n_vertices) *o.n_vertices = ctx->h_ctl->totals[0];
            if (o.n_quads) *o.n_quads = ctx->h_ctl->totals[1];
            if (o.h_results) std::copy(stage_results(b), stage_results(b) + n, o.h_results);
            return ctl_status(ctx->h_ctl);
        }
        // sizing: the totals and the per-volume offsets are final after the scan
        CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaMemcpyAsync(stage_results(b), d_res, sizeof(dmc_batch_result) * (size_t)n, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        stats_from_ctl(ctx);
        if (ctx->h_ctl->err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
        const uint64_t V = ctx->h_ctl->totals[0], Q = ctx->h_ctl->totals[1];
        if (o.n_vertices) *o.n_vertices = V;
        if (o.n_quads) *o.n_quads = Q;
        if (V >= 0xFFFFFFFFull || Q >= 0xFFFFFFFFull) return DMC_ERR_OUTPUT_OVERFLOW;
        if (o.h_results) std::copy(stage_results(b), stage_results(b) + n, o.h_results);
        return DMC_OK;
    }
    CUDA_TRY(cudaEventRecord(b.done, st));
    b.in_flight = true;
    b.n_inflight = n;
    return DMC_OK;
}

static dmc_status stream_state(BatchState &b)
{
    using namespace brick;
    if (b.h_snap) return DMC_OK;
    CUDA_TRY(cudaStreamCreateWithFlags(&b.s_in, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&b.s_out, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&b.ev_start, cudaEventDisableTiming));
    for (int i = 0; i < kMaxSlabs; ++i) {
        CUDA_TRY(cudaEventCreateWithFlags(&b.ev_in[i], cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&b.ev_tot[i], cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&b.ev_emit[i], cudaEventDisableTiming));
    }
    unsigned long long *h = nullptr;
    CUDA_TRY(cudaHostAlloc((void **)&h, 4 * sizeof(unsigned long long) * kMaxSlabs, cudaHostAllocMapped));
    b.h_snap = h;
    CUDA_TRY(cudaHostGetDevicePointer((void **)&b.d_snap, h, 0));
    return DMC_OK;
}

template <class T>
static void launch_sweep(Ctx *ctx, BatchState &b, bool emit, brick::BrickRange r, const brick::EmitOut &eo,
                         uint32_t *ticket, cudaStream_t st)
{
    using namespace brick;
    const uint32_t grp = std::is_same<T, float>::value ? 0 : 1;
    if (emit)
        brick_sweep<T, true><<<sweep_blocks(b, grp, true, r.cnt, false), 32 * NWB_EMIT, kEmitSmem, st>>>(
            b.d_plan, grp, r, ctx->d_tab, nullptr, eo, b.spill, b.cells, ticket, ctx->d_ctl->counters, &ctx->d_ctl->err);
    else
        brick_sweep<T, false><<<sweep_blocks(b, grp, false, r.cnt, false), 32 * NWB_COUNT, kCountSmem, st>>>(
            b.d_plan, grp, r, ctx->d_tab, b.seg_cnt, EmitOut{}, b.spill, b.cells, ticket, ctx->d_ctl->counters, &ctx->d_ctl->err);
}

// Host volume to host mesh in z slabs, so that the upload of later slabs,
// the sweeps of the current ones and the download of finished ones overlap
// (one copy stream each way; the sweeps on st).  Slab i is a run of whole
// z bricks, cell planes [z_i, z_i+1).  Its count sweep runs once the point
// planes up to z_i+1 + 1 are on the device (the 2B/3B test of its last plane
// reads one plane further), its scan continues the running totals, and its
// emit sweep follows the next slab's count and scan (the quads of its last
// plane reference cells of the next plane).  The host reads the totals after
// each slab's scan and downloads that slab's vertex and quad ranges once its
// emit sweep is done.  The mesh equals the unstreamed one bit for bit: same
// bricks, same segment order, the same scan in pieces.
dmc_status brick_run_streamed(Ctx *ctx, const ExtractArgs &a, const StreamIO &io, uint32_t slabs, bool *dev_short,
                              cudaStream_t st)
{
    NvtxRange nvtx("dmc streamed extraction");
    using namespace brick;
    *dev_short = false;
    BatchState *bp = nullptr;
    dmc_status s = batch_state(ctx, &bp);
    if (s != DMC_OK) return s;
    BatchState &b = *bp;
    if (b.in_flight) return DMC_ERR_INVALID_ARG;
    b.shard_ready = false;          // this call replaces a sharded count's plan
    if ((s = stream_state(b)) != DMC_OK) return s;
    BrickItem it;
    it.data = a.vol; it.dtype = a.dtype; it.pts = a.pts; it.cells = a.cells; it.iso = a.iso; it.mn = a.mn; it.rng = a.rng;
    uint64_t nb[2] = {0, 0};
    if ((s = stage_plan(ctx, b, &it, 1, nb)) != DMC_OK) return s;
    BatchHead *head = (BatchHead *)b.h_stage;
    const Geom g = *(const Geom *)(head + 1);
    const bool f32 = a.dtype == DMC_F32;
    // Every slab but the last spans at least two cell planes: the emit sweep
    // of slab i reads the masks of plane z_i+1 + 1, which the count sweep of
    // slab i+1 stores only if that plane lies in slab i+1.
    const uint32_t max_slabs = g.zc >= 2 ? g.nzb : g.nzb / 2;
    const uint32_t S = std::max<uint32_t>(1u, std::min<uint32_t>(std::min<uint32_t>(slabs, max_slabs), (uint32_t)kMaxSlabs));
    const uint64_t bricks_xy = (uint64_t)g.nxs * g.nyb, segs_z = (uint64_t)a.cells.y * g.nxs;
    uint32_t zb[kMaxSlabs + 1], z[kMaxSlabs + 1];
    uint64_t toff[kMaxSlabs + 1];
    // Slab sizes ramp up and down (weights 1, 2, 3, 4, ..., 4, 3, 2, 1): the
    // first slabs are uploaded and the last ones downloaded while the link
    // carries nothing the other way, so they are kept short.
    const uint32_t minb = g.zc >= 2 ? 1u : 2u;
    uint64_t wsum = 0, wc[kMaxSlabs + 1];
    wc[0] = 0;
    for (uint32_t i = 0; i < S; ++i) wc[i + 1] = (wsum += std::min<uint32_t>(std::min(i + 1, S - i), 4u));
    zb[0] = 0;
    zb[S] = g.nzb;
    for (uint32_t i = 1; i < S; ++i)
        zb[i] = (uint32_t)std::min<uint64_t>(std::max<uint64_t>((uint64_t)g.nzb * wc[i] / wsum, zb[i - 1] + minb),
                                             (uint64_t)g.nzb - (uint64_t)(S - i) * minb);
    for (uint32_t i = 0; i <= S; ++i) z[i] = std::min<uint32_t>(zb[i] * g.zc, a.cells.z);
    toff[0] = 0;
    for (uint32_t i = 0; i < S; ++i) toff[i + 1] = toff[i] + ((uint64_t)(z[i + 1] - z[i]) * segs_z + SCAN_TILE - 1) / SCAN_TILE;
    head->n_tiles = (uint32_t)toff[S];   // the prep kernel clears every slab's tiles

    // uploads: slab i brings the point planes up to z_i+1 + 1 not brought before
    const uint64_t plane = (uint64_t)a.pts.x * a.pts.y * (f32 ? 4u : 2u);
    uint8_t *dvol = (uint8_t *)const_cast<void *>(a.vol);
    const uint8_t *hvol = (const uint8_t *)io.h_vol;
    CUDA_TRY(cudaEventRecord(ctx->ev0, st));
    CUDA_TRY(cudaEventRecord(b.ev_start, st));
    CUDA_TRY(cudaStreamWaitEvent(b.s_in, b.ev_start, 0));   // earlier work on st may still read the device volume
    CUDA_TRY(cudaStreamWaitEvent(b.s_out, b.ev_start, 0));
    uint64_t p0 = 0;
    for (uint32_t i = 0; i < S; ++i) {
        const uint64_t p1 = i + 1 == S ? a.pts.z - 1ull : std::min<uint64_t>((uint64_t)z[i + 1] + 1, a.pts.z - 1ull);
        if (p0 <= p1)
            CUDA_TRY(cudaMemcpyAsync(dvol + p0 * plane, hvol + p0 * plane, (p1 - p0 + 1) * plane, cudaMemcpyHostToDevice, b.s_in));
        CUDA_TRY(cudaEventRecord(b.ev_in[i], b.s_in));
        p0 = std::max(p0, p1 + 1);
    }

    CUDA_TRY(cudaMemcpyAsync(b.d_plan, b.h_stage, b.plan_bytes, cudaMemcpyHostToDevice, st));
    batch_prep<<<2 * ctx->num_sms, 256, 0, st>>>(b.d_plan, b.tiles, b.tickets, ctx->d_ctl);
    CUDA_TRY(cudaGetLastError());
    EmitOut eo;
    eo.seg_off = b.seg_off; eo.verts = a.verts; eo.vcap = a.vcap; eo.quads = a.quads; eo.qcap = a.qcap; eo.tris = a.tris;
    auto range = [&](uint32_t i) { return BrickRange{(uint32_t)(zb[i] * bricks_xy), (uint32_t)((zb[i + 1] - zb[i]) * bricks_xy)}; };
    for (uint32_t i = 0; i <= S; ++i) {
        if (i < S) {
            CUDA_TRY(cudaStreamWaitEvent(st, b.ev_in[i], 0));
            if (f32) launch_sweep<float>(ctx, b, false, range(i), eo, &b.tickets[4 + 3 * i], st);
            else launch_sweep<uint16_t>(ctx, b, false, range(i), eo, &b.tickets[4 + 3 * i], st);
            CUDA_TRY(cudaGetLastError());
            ScanCtl ctl;
            ctl.tiles = b.tiles + toff[i]; ctl.ticket = &b.tickets[4 + 3 * i + 2]; ctl.err = &ctx->d_ctl->err;
            ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = 0; ctl.carry = ctx->d_ctl->totals;
            const uint64_t nt = toff[i + 1] - toff[i];
            seg_scan<<<(int)std::max<uint64_t>(1, std::min<uint64_t>(2ull * ctx->num_sms, nt)), SCAN_NT, 0, st>>>(
                b.d_plan, b.seg_cnt, ctl, b.seg_off, (uint64_t)z[i] * segs_z, (uint64_t)(z[i + 1] - z[i]) * segs_z);
            snap_totals<<<1, 32, 0, st>>>(ctx->d_ctl, b.d_snap + 4 * i);
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaEventRecord(b.ev_tot[i], st));
        }
        if (i >= 1) {
            if (f32) launch_sweep<float>(ctx, b, true, range(i - 1), eo, &b.tickets[4 + 3 * (i - 1) + 1], st);
            else launch_sweep<uint16_t>(ctx, b, true, range(i - 1), eo, &b.tickets[4 + 3 * (i - 1) + 1], st);
            CUDA_TRY(cudaGetLastError());
            CUDA_TRY(cudaEventRecord(b.ev_emit[i - 1], st));
        }
    }
    CUDA_TRY(cudaEventRecord(ctx->ev1, st));
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));

    // downloads, slab by slab, as the totals come in
    uint64_t pv = 0, pq = 0;
    bool host_short = false, stop = false;
    for (uint32_t i = 0; i < S; ++i) {
        CUDA_TRY(cudaEventSynchronize(b.ev_tot[i]));
        const volatile unsigned long long *sn = b.h_snap + 4 * i;
        const uint64_t tv = sn[0], tq = sn[1];
        if (sn[2]) stop = true;
        if (tv > a.vcap || tq > a.qcap) { *dev_short = true; stop = true; }
        if (tv > io.vcap || tq > io.qcap) { host_short = true; stop = true; }
        if (!stop && (tv > pv || tq > pq)) {
            CUDA_TRY(cudaStreamWaitEvent(b.s_out, b.ev_emit[i], 0));
            if (tv > pv)
                CUDA_TRY(cudaMemcpyAsync(io.hv + 3 * pv, a.verts + 3 * pv, 12 * (tv - pv), cudaMemcpyDeviceToHost, b.s_out));
            if (tq > pq) {
                if (io.hq)
                    CUDA_TRY(cudaMemcpyAsync(io.hq + 4 * pq, a.quads + 4 * pq, 16 * (tq - pq), cudaMemcpyDeviceToHost, b.s_out));
                if (io.ht)
                    CUDA_TRY(cudaMemcpyAsync(io.ht + 6 * pq, a.tris + 6 * pq, 24 * (tq - pq), cudaMemcpyDeviceToHost, b.s_out));
            }
        }
        pv = tv; pq = tq;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    CUDA_TRY(cudaStreamSynchronize(b.s_out));
    event_ms(&ctx->stats.device_ms, ctx->ev0, ctx->ev1);
    stats_from_ctl(ctx);
    if (ctx->h_ctl->err & DEV_ERR_OVERFLOW) *dev_short = true;
    if (*dev_short) return DMC_ERR_OUTPUT_OVERFLOW;
    if ((s = ctl_status(ctx->h_ctl)) != DMC_OK) return s;
    return host_short ? DMC_ERR_OUTPUT_OVERFLOW : DMC_OK;
}

// Sharded extraction of one volume across ranks in z slabs (the volume's
// cell planes [z_begin, z_end) on this rank).  it.pts / it.cells are the
// whole volume's; it.data points to this rank's copy of the point planes
// from plane0 on, which must cover [z_begin - 1, z_end + 3) within the
// volume: one plane below for the 2B/3B test of the first cell plane; above,
// the next shard's first cell plane (whose offsets the quads of the last
// plane reference) with its own 2B/3B test.
//
// Phase 1 (brick_shard_count): the count sweep over the shard's bricks, a
// plane-limited count of the next shard's first plane (no counters), and
// the scan of the shard's segments plus that plane, from zero.  The shard's
// totals are the offsets at the next shard's first plane.
// Phase 2 (brick_shard_emit): with the vertex offset of all earlier shards
// (an exclusive scan of the totals across ranks), the emit sweep writes the
// shard's vertices and quads at local positions, quad indices made global.
// In rank order the parts form the unsharded mesh: the same bricks, the same
// segment order, the same scan in pieces.
dmc_status brick_shard_count(Ctx *ctx, const BrickItem &item, uint32_t plane0, uint32_t z_begin, uint32_t z_end,
                             uint64_t *V, uint64_t *Q, cudaStream_t st)
{
    using namespace brick;
    BatchState *bp = nullptr;
    dmc_status s = batch_state(ctx, &bp);
    if (s != DMC_OK) return s;
    BatchState &b = *bp;
    if (b.in_flight) return DMC_ERR_INVALID_ARG;
    b.shard_ready = false;
    const uint3 cells = item.cells;
    if (z_begin >= z_end || z_end > cells.z) return DMC_ERR_INVALID_ARG;
    // bricks of this shard's size, then as deep as both shard boundaries allow
    BrickItem shard = item;
    shard.cells.z = z_end - z_begin;
    uint32_t zc = pick_zc(ctx, b, &shard, 1);
    while (zc > 1 && (z_begin % zc != 0 || (z_end != cells.z && z_end % zc != 0))) zc >>= 1;
    // the kernels index the volume by global plane: shift the base by plane0 planes
    const uint64_t plane_bytes = (uint64_t)item.pts.x * item.pts.y * (item.dtype == DMC_F32 ? 4u : 2u);
    BrickItem it = item;
    it.data = reinterpret_cast<const void *>(reinterpret_cast<uintptr_t>(item.data) - (uintptr_t)(plane0 * plane_bytes));
    uint64_t nb[2] = {0, 0};
    if ((s = stage_plan(ctx, b, &it, 1, nb, zc)) != DMC_OK) return s;
    BatchHead *head = (BatchHead *)b.h_stage;
    const Geom &g = *(const Geom *)(head + 1);
    const int grp = it.dtype == DMC_F32 ? 0 : 1;
    const uint64_t bxy = (uint64_t)g.nxs * g.nyb, segs_z = (uint64_t)cells.y * g.nxs;
    const uint32_t zb0 = z_begin / zc, zb1 = z_end == cells.z ? g.nzb : z_end / zc;
    const bool halo = z_end < cells.z;

    CUDA_TRY(cudaEventRecord(ctx->ev0, st));
    CUDA_TRY(cudaMemcpyAsync(b.d_plan, b.h_stage, b.plan_bytes, cudaMemcpyHostToDevice, st));
    batch_prep<<<2 * ctx->num_sms, 256, 0, st>>>(b.d_plan, b.tiles, b.tickets, ctx->d_ctl);
    CUDA_TRY(cudaGetLastError());
    EmitOut none{};
    const BrickRange own{(uint32_t)(zb0 * bxy), (uint32_t)((zb1 - zb0) * bxy)};
    if (grp == 0) launch_sweep<float>(ctx, b, false, own, none, &b.tickets[0], st);
    else launch_sweep<uint16_t>(ctx, b, false, own, none, &b.tickets[1], st);
    if (halo) {
        BrickRange next{(uint32_t)(zb1 * bxy), (uint32_t)bxy};
        next.zlim = z_end + 1;
        next.flags = kNoStats;
        if (grp == 0) launch_sweep<float>(ctx, b, false, next, none, &b.tickets[4], st);
        else launch_sweep<uint16_t>(ctx, b, false, next, none, &b.tickets[4], st);
    }
    CUDA_TRY(cudaGetLastError());
    ScanCtl ctl;
    ctl.tiles = b.tiles; ctl.ticket = &b.tickets[5]; ctl.err = &ctx->d_ctl->err;
    ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = 0;
    const uint64_t seg0 = (uint64_t)z_begin * segs_z, nseg = (uint64_t)(z_end - z_begin + (halo ? 1 : 0)) * segs_z;
    const uint64_t nt = (nseg + SCAN_TILE - 1) / SCAN_TILE;
    seg_scan<<<(int)std::max<uint64_t>(1, std::min<uint64_t>(2ull * ctx->num_sms, nt)), SCAN_NT, 0, st>>>(
        b.d_plan, b.seg_cnt, ctl, b.seg_off, seg0, nseg);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    // the shard's totals: the offsets where the next shard's first plane starts
    uint2 *h_off = reinterpret_cast<uint2 *>(stage_results(b));
    if (halo)
        CUDA_TRY(cudaMemcpyAsync(h_off, b.seg_off + (uint64_t)z_end * segs_z, sizeof(uint2), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(ctx->ev1, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    stats_from_ctl(ctx);
    const uint32_t err = ctx->h_ctl->err;
    if (err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    if (err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    const uint64_t tv = halo ? h_off->x : ctx->h_ctl->totals[0], tq = halo ? h_off->y : ctx->h_ctl->totals[1];
    ctx->stats.n_vertices = tv;
    ctx->stats.n_quads = tq;
    if (V) *V = tv;
    if (Q) *Q = tq;
    if (ctx->h_ctl->totals[0] >= 0xFFFFFFFFull || ctx->h_ctl->totals[1] >= 0xFFFFFFFFull) return DMC_ERR_OUTPUT_OVERFLOW;
    b.shard_ready = true;
    b.sh_scratch_gen = ctx->scratch_gen;
    b.sh_grp = grp; b.sh_zb0 = zb0; b.sh_zb1 = zb1; b.sh_bxy = bxy;
    return DMC_OK;
}

dmc_status brick_shard_emit(Ctx *ctx, uint64_t vertex_offset, const BrickOut &o, cudaStream_t st)
{
    using namespace brick;
    BatchState *b = ctx->batch;
    // the count phase must be the context's last brick call, with its scratch still in place
    if (!b || !b->shard_ready || b->in_flight || b->sh_scratch_gen != ctx->scratch_gen) return DMC_ERR_INVALID_ARG;
    // quad indices: local vertex index + vertex_offset (the emit subtracts vbase)
    Geom *hg = (Geom *)((BatchHead *)b->h_stage + 1);
    hg->vbase = (uint32_t)(0u - (uint32_t)vertex_offset);
    Geom *dg = (Geom *)(b->d_plan + 1);
    CUDA_TRY(cudaEventRecord(ctx->ev0, st));
    CUDA_TRY(cudaMemcpyAsync(&dg->vbase, &hg->vbase, sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    EmitOut eo;
    eo.seg_off = b->seg_off; eo.verts = o.verts; eo.vcap = o.vcap; eo.quads = o.quads; eo.qcap = o.qcap; eo.tris = o.tris;
    const BrickRange own{(uint32_t)(b->sh_zb0 * b->sh_bxy), (uint32_t)((b->sh_zb1 - b->sh_zb0) * b->sh_bxy)};
    if (b->sh_grp == 0) launch_sweep<float>(ctx, *b, true, own, eo, &b->tickets[2], st);
    else launch_sweep<uint16_t>(ctx, *b, true, own, eo, &b->tickets[3], st);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaEventRecord(ctx->ev1, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    b->shard_ready = false;      // the emit sweep consumed the tickets
    const uint32_t err = ctx->h_ctl->err;
    if (err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    if (err & DEV_ERR_OVERFLOW) return DMC_ERR_OUTPUT_OVERFLOW;
    if (err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    return DMC_OK;
}

dmc_status brick_wait(Ctx *ctx, dmc_batch_result *h_results, uint64_t *n_vertices, uint64_t *n_quads)
{
    BatchState *b = ctx->batch;
    if (!b || !b->in_flight) return DMC_ERR_INVALID_ARG;
    b->in_flight = false;
    CUDA_TRY(cudaEventSynchronize(b->done));
    stats_from_ctl(ctx);
    if (n_vertices) *n_vertices = ctx->h_ctl->totals[0];
    if (n_quads) *n_quads = ctx->h_ctl->totals[1];
    if (h_results) std::copy(stage_results(*b), stage_results(*b) + b->n_inflight, h_results);
    return ctl_status(ctx->h_ctl);
}

dmc_status brick_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st)
{
    BrickItem it;
    it.data = a.vol; it.dtype = a.dtype; it.pts = a.pts; it.cells = a.cells; it.iso = a.iso; it.mn = a.mn; it.rng = a.rng;
    BrickOut o{};
    o.verts = a.verts; o.vcap = a.vcap; o.quads = a.quads; o.qcap = a.qcap; o.tris = a.tris;
    o.mode = BATCH_SYNC; o.sizing_only = a.sizing_only;
    o.n_vertices = a.n_vertices; o.n_quads = a.n_quads;
    return brick_extract(ctx, &it, 1, o, st);
}

}  // namespace dmc
