// Internal host-side declarations shared by the extraction paths.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include "../../include/dmc_gb300.h"
#include "dmc_device.cuh"

namespace dmc {

// A named NVTX range over a host scope, for profiler timelines (Nsight
// Systems, ncu's NVTX filters).  Without a tool attached it costs a call.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

#define CUDA_TRY(expr)                                              \
    do {                                                            \
        cudaError_t _e = (expr);                                    \
        if (_e != cudaSuccess) {                                    \
            ::dmc::set_last_cuda_error(_e);                         \
            return _e == cudaErrorMemoryAllocation ? DMC_ERR_OOM : DMC_ERR_CUDA; \
        }                                                           \
    } while (0)

void set_last_cuda_error(cudaError_t e);

// Small control block in device memory, mirrored to pinned host memory.
struct DevCtl {
    uint32_t ticket;                   // look-back tile ticket
    uint32_t err;                      // DEV_ERR_* bits
    unsigned long long totals[2];      // vertices, quads
    unsigned long long counters[4];    // active cells, lut2 cells, dropped quads, spare
    uint32_t ticket2;                  // second ticket (brick work queue)
    uint32_t pad[7];
};

struct BatchState;

struct Ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evk[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};   // per-kernel timing (brick path)
    int evk_used = 0;                   // 1: count and scan timed, 2: emit timed too
    void *scratch = nullptr;           // grow-only device scratch
    size_t scratch_bytes = 0;
    DevCtl *d_ctl = nullptr;
    DevCtl *h_ctl = nullptr;           // pinned
    void *d_vol = nullptr;             // staging for host volumes (grow-only)
    uint64_t scratch_gen = 0;          // bumped whenever scratch moves (captured graphs hold its addresses)
    uint32_t brick_zc = 0;             // planes per brick (0: automatic)
    uint32_t stream_slabs = 0;         // host extraction in z slabs: 0 automatic, 1 never, n >= 2 n slabs
    uint32_t fail_allocs = 0;          // test hook: device allocations still to fail (DMC_OPT_FAIL_ALLOCS)
    BatchState *batch = nullptr;
    bool batch_pending = false;        // an asynchronous batch awaits dmc_batch_wait
    size_t d_vol_bytes = 0;
    DeviceTables *d_tab = nullptr;     // lookup tables in device memory
    int algo = DMC_ALGO_AUTO;
    dmc_stats stats{};
};

// Cells of a volume, (nx-1)(ny-1)(nz-1) from its cell counts per axis; false
// when the product does not fit 64 bits.
inline bool cell_count(uint3 c, uint64_t *n)
{
    uint64_t xy;
    return !__builtin_mul_overflow((uint64_t)c.x, (uint64_t)c.y, &xy) && !__builtin_mul_overflow(xy, (uint64_t)c.z, n);
}

struct ExtractArgs {
    const void *vol;
    dmc_dtype dtype;
    uint3 pts, cells;
    uint64_t n_cells;
    float iso;
    float3 mn, rng;
    float *verts; uint64_t vcap;
    uint32_t *quads; uint64_t qcap;
    uint32_t *tris;
    uint64_t *n_vertices, *n_quads;
    bool sizing_only;                  // count only: report totals, write no mesh
    uint32_t num_smooth;               // smoothing iterations (simple path; needs the quad buffer)
};

dmc_status ctx_reserve_scratch(Ctx *ctx, size_t bytes);

// Milliseconds between two recorded events into *ms (unchanged when the
// query fails, e.g. an event that was never recorded).  A failed query's
// error is cleared, so that it cannot surface in a later launch check.
inline void event_ms(float *ms, cudaEvent_t a, cudaEvent_t b)
{
    float v = 0.f;
    if (cudaEventElapsedTime(&v, a, b) == cudaSuccess) *ms = v;
    else (void)cudaGetLastError();
}

// One volume of a brick-path extraction.
struct BrickItem {
    const void *data;          // device samples
    dmc_dtype dtype;
    uint3 pts, cells;
    float iso;
    float3 mn, rng;
};

enum BatchMode { BATCH_SYNC = 0, BATCH_ASYNC = 1, BATCH_GRAPH = 2 };

struct BrickOut {
    float *verts; uint64_t vcap;
    uint32_t *quads; uint64_t qcap;
    uint32_t *tris;
    dmc_batch_result *d_results;   // per volume, device (may be NULL)
    dmc_batch_result *h_results;   // per volume, host (may be NULL; BATCH_SYNC only)
    uint64_t *n_vertices, *n_quads; // totals (host; BATCH_SYNC only)
    BatchMode mode;
    bool sizing_only;              // BATCH_SYNC: stop after the count
};

// State of the batch pipeline of a context (scratch layout, pinned staging,
// cached graph, the batch in flight).  Defined with the brick kernels.
void batch_state_free(Ctx *ctx);

dmc_status brick_extract(Ctx *ctx, const BrickItem *items, uint32_t n, const BrickOut &o, cudaStream_t st);

// Host side of a streamed extraction: the host volume, and the caller's host
// output buffers with their capacities (vertices, quads; triangles may be null).
struct StreamIO {
    const void *h_vol;
    float *hv; uint64_t vcap;
    uint32_t *hq; uint64_t qcap;
    uint32_t *ht;
};
// Streamed host extraction in z slabs (a.vol: the device copy of the volume,
// a.verts/quads/tris: device output buffers).  DMC_ERR_OUTPUT_OVERFLOW with
// *dev_short set means the device buffers were too small (nothing complete was
// downloaded; the totals are in the context's stats).
dmc_status brick_run_streamed(Ctx *ctx, const ExtractArgs &a, const StreamIO &io, uint32_t slabs, bool *dev_short,
                              cudaStream_t st);
// Sharded extraction (dmc_shard_count / dmc_shard_emit): item describes the
// whole volume, item.data this rank's point planes from plane0 on.
dmc_status brick_shard_count(Ctx *ctx, const BrickItem &item, uint32_t plane0, uint32_t z_begin, uint32_t z_end,
                             uint64_t *V, uint64_t *Q, cudaStream_t st);
dmc_status brick_shard_emit(Ctx *ctx, uint64_t vertex_offset, const BrickOut &o, cudaStream_t st);
// Completes an asynchronous batch: waits for it and checks its status.
dmc_status brick_wait(Ctx *ctx, dmc_batch_result *h_results, uint64_t *n_vertices, uint64_t *n_quads);
dmc_status upload_tables(Ctx *ctx);
void fill_tables(DeviceTables &h);   // host copy of the lookup tables

dmc_status simple_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st);
dmc_status brick_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st);
bool brick_supports(const ExtractArgs &a);

}  // namespace dmc
