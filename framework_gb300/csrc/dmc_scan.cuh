// Single-pass exclusive scan with decoupled look-back, for pairs of counts
// (vertices, quads).  This replaces the reference's Thrust reduce + exclusive
// scan pairs (dmc.cu:1071-1087, 2092-2098, 2133-2139, 2178-2183): one pass
// over the data, no host round trip for the totals.
//
// Each tile publishes its aggregate, then walks back over its predecessors
// (32 at a time, one warp) until it meets a tile whose inclusive prefix is
// known.  Tiles are numbered by an atomic ticket in the order blocks start, so
// a tile only ever waits on tiles that are already running.  Every wait is
// bounded; on timeout the kernel records DEV_ERR_TIMEOUT and carries on with a
// zero prefix, and the host reports DMC_ERR_TIMEOUT.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "dmc_device.cuh"

namespace dmc {

struct TileState {
    uint32_t flag;        // 0 empty, 1 aggregate published, 2 inclusive published
    uint32_t agg_v, agg_q;
    uint32_t pad;
    unsigned long long inc_v, inc_q;
};

struct ScanCtl {
    TileState *tiles;
    uint32_t *ticket;
    uint32_t *err;
    unsigned long long *totals;   // [0] vertices, [1] quads (written by the last tile)
    uint32_t n_tiles;
    // optional carry-in: the scan continues from these totals (read by tile 0
    // only, before the last tile overwrites them), so that consecutive
    // launches over consecutive ranges form one scan
    const unsigned long long *carry = nullptr;
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

constexpr uint32_t kSpinLimit = 1u << 20;   // ~ 1M polls with back-off, far above any real wait

// Claim a tile number in start order.  Call from all threads; uses smem slot.
__device__ __forceinline__ uint32_t claim_tile(uint32_t *ticket, uint32_t *s_slot)
{
    if (threadIdx.x == 0) *s_slot = atomicAdd(ticket, 1u);
    __syncthreads();
    uint32_t t = *s_slot;
    __syncthreads();
    return t;
}

// Given the tile's aggregates (valid in thread 0), returns in every thread the
// exclusive prefix of the tile.  s_ex must point to 2 x u64 of shared memory.
__device__ __forceinline__ void tile_prefix(const ScanCtl &c, uint32_t tile, uint32_t agg_v, uint32_t agg_q,
                                            unsigned long long *s_ex)
{
    TileState *ts = c.tiles;
    if (threadIdx.x == 0) {
        ts[tile].agg_v = agg_v;
        ts[tile].agg_q = agg_q;
        if (tile == 0) {
            ts[tile].inc_v = (c.carry ? c.carry[0] : 0ull) + agg_v;
            ts[tile].inc_q = (c.carry ? c.carry[1] : 0ull) + agg_q;
            __threadfence();
            st_release(&ts[tile].flag, 2u);
        } else {
            __threadfence();
            st_release(&ts[tile].flag, 1u);
        }
    }
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        unsigned long long ex_v = 0, ex_q = 0;
        if (tile == 0 && c.carry) { ex_v = c.carry[0]; ex_q = c.carry[1]; }
        if (tile > 0) {
            long long base = (long long)tile - 1;
            bool done = false;
            while (!done) {
                long long idx = base - lane;
                uint32_t flag = 2;
                unsigned long long vv = 0, vq = 0;
                if (idx >= 0) {
                    uint32_t spins = 0;
                    flag = ld_acquire(&ts[idx].flag);
                    while (flag == 0) {
                        if (++spins > kSpinLimit) { atomicOr(c.err, DEV_ERR_TIMEOUT); flag = 2; break; }
                        __nanosleep(spins < 64 ? 32 : 256);
                        flag = ld_acquire(&ts[idx].flag);
                    }
                    if (flag == 2) {
                        vv = *(volatile unsigned long long *)&ts[idx].inc_v;
                        vq = *(volatile unsigned long long *)&ts[idx].inc_q;
                    } else {
                        vv = *(volatile uint32_t *)&ts[idx].agg_v;
                        vq = *(volatile uint32_t *)&ts[idx].agg_q;
                    }
                }
                unsigned incl = __ballot_sync(0xffffffffu, flag == 2);
                int stop = incl ? __ffs(incl) - 1 : 32;   // nearest predecessor with inclusive prefix
                if (lane > stop) { vv = 0; vq = 0; }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    vv += __shfl_xor_sync(0xffffffffu, vv, o);
                    vq += __shfl_xor_sync(0xffffffffu, vq, o);
                }
                ex_v += vv; ex_q += vq;
                if (incl) done = true;
                base -= 32;
            }
        }
        if (lane == 0) {
            s_ex[0] = ex_v; s_ex[1] = ex_q;
            if (tile > 0) {
                ts[tile].inc_v = ex_v + agg_v;
                ts[tile].inc_q = ex_q + agg_q;
                __threadfence();
                st_release(&ts[tile].flag, 2u);
            }
            if (tile == c.n_tiles - 1) {
                c.totals[0] = ex_v + agg_v;
                c.totals[1] = ex_q + agg_q;
            }
        }
    }
    __syncthreads();
}

// Block-wide exclusive scan of a 64-bit value (two packed 32-bit counters
// cannot overflow inside one block).  Returns the exclusive prefix of the
// thread and, through *total, the block sum.  s_warp: NT/32 u64 of smem.
template <int NT>
__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long x, unsigned long long *s_warp,
                                                                   unsigned long long *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < NT / 32 ? s_warp[lane] : 0ull;
        unsigned long long wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < NT / 32) s_warp[lane] = wi - w;
        if (lane == NT / 32 - 1) s_warp[NT / 32] = wi;
    }
    __syncthreads();
    unsigned long long res = s_warp[warp] + inc - x;
    *total = s_warp[NT / 32];
    __syncthreads();
    return res;
}

}  // namespace dmc
