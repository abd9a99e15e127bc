// Internal host-side declarations shared by the extraction paths.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "../../include/dmc_gb300.h"
#include "dmc_device.cuh"

namespace dmc {

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
    size_t d_vol_bytes = 0;
    DeviceTables *d_tab = nullptr;     // lookup tables in device memory
    int algo = DMC_ALGO_AUTO;
    dmc_stats stats{};
};

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
};

dmc_status ctx_reserve_scratch(Ctx *ctx, size_t bytes);
dmc_status upload_tables(Ctx *ctx);

dmc_status simple_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st);
dmc_status brick_run(Ctx *ctx, const ExtractArgs &a, cudaStream_t st);
bool brick_supports(const ExtractArgs &a);

}  // namespace dmc
