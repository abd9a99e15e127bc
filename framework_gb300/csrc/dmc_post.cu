// Opt-in mesh post-processing (dmc_compact_mesh): drop every vertex that no
// quad references and renumber the index buffers.  In a dual-contouring mesh
// the quads connect dual vertices only; the edge crossings (dmc.cu:1468-1514)
// exist to place the dual vertices, so a consumer that needs only the surface
// can drop them.  The output no longer has the reference's vertex numbering,
// which is why this is a separate call and never part of the extraction.
//
// Three launches: mark the referenced vertices, one look-back scan over the
// marks that also gathers the kept vertices to their new places, and the
// renumbering of the quads (and triangles) in place.
#include "dmc_scan.cuh"
#include "dmc_internal.h"

namespace dmc {

constexpr int kPostThreads = 256, kPostItems = 8, kPostTile = kPostThreads * kPostItems;

__global__ void __launch_bounds__(kPostThreads) post_mark(const uint4 *__restrict__ quads, uint64_t n_quads,
                                                          uint64_t n_vertices, uint8_t *__restrict__ used,
                                                          uint32_t *err)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_quads; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint4 q = quads[i];
        const uint32_t id[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (id[k] < n_vertices) used[id[k]] = 1;
            else atomicOr(err, DEV_ERR_BOUNDS);
        }
    }
}

// new index of every vertex (exclusive count of kept vertices before it);
// kept vertices are copied to their new place on the way
__global__ void __launch_bounds__(kPostThreads) post_scan_gather(const uint8_t *__restrict__ used, uint64_t n,
                                                                 ScanCtl ctl, uint32_t *__restrict__ newidx,
                                                                 const float *__restrict__ vin,
                                                                 float *__restrict__ vout)
{
    __shared__ uint32_t s_slot;
    __shared__ unsigned long long s_warp[kPostThreads / 32 + 1];
    __shared__ unsigned long long s_ex[2];
    const uint32_t tile = claim_tile(ctl.ticket, &s_slot);
    const uint64_t first = (uint64_t)tile * kPostTile + (uint64_t)threadIdx.x * kPostItems;
    uint32_t u[kPostItems], sum = 0;
#pragma unroll
    for (int i = 0; i < kPostItems; ++i) {
        u[i] = first + i < n ? used[first + i] : 0u;
        sum += u[i];
    }
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan<kPostThreads>((unsigned long long)sum, s_warp, &tot);
    tile_prefix(ctl, tile, (uint32_t)tot, 0u, s_ex);
    uint64_t at = s_ex[0] + ex;
#pragma unroll
    for (int i = 0; i < kPostItems; ++i) {
        const uint64_t v = first + i;
        if (v < n) {
            newidx[v] = (uint32_t)at;
            if (u[i]) {
                vout[3 * at + 0] = vin[3 * v + 0];
                vout[3 * at + 1] = vin[3 * v + 1];
                vout[3 * at + 2] = vin[3 * v + 2];
            }
        }
        at += u[i];
    }
}

__global__ void __launch_bounds__(kPostThreads) post_remap(uint32_t *__restrict__ idx, uint64_t n,
                                                           const uint32_t *__restrict__ newidx, uint64_t n_vertices)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = idx[i];
        if (v < n_vertices) idx[i] = newidx[v];
    }
}

}  // namespace dmc

using namespace dmc;

struct dmc_ctx;
namespace dmc { Ctx *ctx_of(dmc_ctx *ctx); }

extern "C" dmc_status dmc_compact_mesh(dmc_ctx *handle, const float *d_vertices, uint64_t n_vertices,
                                       uint32_t *d_quads, uint64_t n_quads, uint32_t *d_triangles,
                                       float *d_out_vertices, uint64_t *n_out_vertices, void *stream)
{
    dmc::NvtxRange nvtx("dmc_compact_mesh");
    if (!handle || !n_out_vertices || (n_vertices && (!d_vertices || !d_out_vertices)) || (n_quads && !d_quads))
        return DMC_ERR_INVALID_ARG;
    if (n_vertices >= 0xFFFFFFFFull) return DMC_ERR_UNSUPPORTED;
    // the gather reads vertex v after every earlier tile has written: the
    // output must not overlap the input
    if (n_vertices && d_out_vertices < d_vertices + 3 * n_vertices && d_vertices < d_out_vertices + 3 * n_vertices)
        return DMC_ERR_INVALID_ARG;
    Ctx *ctx = ctx_of(handle);
    if (ctx->batch_pending) return DMC_ERR_INVALID_ARG;
    *n_out_vertices = 0;
    if (n_vertices == 0) return DMC_OK;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    const uint32_t n_tiles = (uint32_t)((n_vertices + kPostTile - 1) / kPostTile);
    size_t off = 0;
    auto carve = [&](size_t bytes) { size_t o = off; off += (bytes + 255) & ~(size_t)255; return o; };
    const size_t o_used = carve(n_vertices), o_new = carve(4 * n_vertices), o_tiles = carve(sizeof(TileState) * n_tiles);
    dmc_status s = ctx_reserve_scratch(ctx, off);
    if (s != DMC_OK) return s;
    uint8_t *base = (uint8_t *)ctx->scratch;
    uint8_t *used = base + o_used;
    uint32_t *newidx = (uint32_t *)(base + o_new);
    TileState *tiles = (TileState *)(base + o_tiles);
    CUDA_TRY(cudaMemsetAsync(used, 0, n_vertices, st));
    CUDA_TRY(cudaMemsetAsync(tiles, 0, sizeof(TileState) * n_tiles, st));
    CUDA_TRY(cudaMemsetAsync(ctx->d_ctl, 0, sizeof(DevCtl), st));
    const int g = ctx->num_sms * 8;
    if (n_quads) post_mark<<<g, kPostThreads, 0, st>>>(reinterpret_cast<const uint4 *>(d_quads), n_quads, n_vertices, used,
                                                       &ctx->d_ctl->err);
    ScanCtl ctl;
    ctl.tiles = tiles; ctl.ticket = &ctx->d_ctl->ticket; ctl.err = &ctx->d_ctl->err;
    ctl.totals = ctx->d_ctl->totals; ctl.n_tiles = n_tiles;
    post_scan_gather<<<n_tiles, kPostThreads, 0, st>>>(used, n_vertices, ctl, newidx, d_vertices, d_out_vertices);
    if (n_quads) post_remap<<<g, kPostThreads, 0, st>>>(d_quads, 4 * n_quads, newidx, n_vertices);
    if (n_quads && d_triangles) post_remap<<<g, kPostThreads, 0, st>>>(d_triangles, 6 * n_quads, newidx, n_vertices);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemcpyAsync(ctx->h_ctl, ctx->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (ctx->h_ctl->err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    if (ctx->h_ctl->err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    *n_out_vertices = ctx->h_ctl->totals[0];
    return DMC_OK;
}
