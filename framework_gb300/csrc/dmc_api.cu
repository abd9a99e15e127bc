// C ABI entry points (include/dmc_gb300.h): context, table upload, host and
// device forms of the extraction.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <new>
#include <thread>
#include "dmc_internal.h"
#include <vector>

namespace dmc {

// The CUDA error behind the last DMC_ERR_CUDA / DMC_ERR_OOM of this thread,
// as the reference's error check prints it before exiting
// (cuda_includes.h:13-19): the error's name and description.
static thread_local char g_last_cuda[256];
void set_last_cuda_error(cudaError_t e)
{
    snprintf(g_last_cuda, sizeof(g_last_cuda), "%s: %s", cudaGetErrorName(e), cudaGetErrorString(e));
}

// The DMC_OPT_FAIL_ALLOCS hook: true while allocations are to fail.
static bool fake_oom(Ctx *ctx)
{
    if (!ctx->fail_allocs) return false;
    --ctx->fail_allocs;
    set_last_cuda_error(cudaErrorMemoryAllocation);   // as the failing cudaMalloc would report
    return true;
}

dmc_status ctx_reserve_scratch(Ctx *ctx, size_t bytes)
{
    if (bytes <= ctx->scratch_bytes) return DMC_OK;
    // Freeing the old scratch invalidates every layout carved from it (the
    // batch plan, captured graphs, a sharded count), also when the new
    // allocation then fails: the generation moves with the free.
    if (ctx->scratch) { cudaFree(ctx->scratch); ctx->scratch = nullptr; ctx->scratch_bytes = 0; ++ctx->scratch_gen; }
    size_t want = bytes + bytes / 8;   // headroom: fewer re-allocations across calls
    if (fake_oom(ctx)) return DMC_ERR_OOM;
    CUDA_TRY(cudaMalloc(&ctx->scratch, want));
    ctx->scratch_bytes = want;
    ++ctx->scratch_gen;
    return DMC_OK;
}

static dmc_status reserve(Ctx *ctx, void **p, size_t *have, size_t bytes)
{
    if (bytes <= *have) return DMC_OK;
    if (*p) { cudaFree(*p); *p = nullptr; *have = 0; }
    size_t want = bytes + bytes / 8 + 256;
    if (fake_oom(ctx)) return DMC_ERR_OOM;
    CUDA_TRY(cudaMalloc(p, want));
    *have = want;
    return DMC_OK;
}

void fill_tables(DeviceTables &h)
{
    memcpy(h.edge_lut[0], DMC_EDGE_LUT1, sizeof(h.edge_lut[0]));
    memcpy(h.edge_lut[1], DMC_EDGE_LUT2, sizeof(h.edge_lut[1]));
    memcpy(h.nvert[0], DMC_NVERT_LUT1, sizeof(h.nvert[0]));
    memcpy(h.nvert[1], DMC_NVERT_LUT2, sizeof(h.nvert[1]));
    memcpy(h.amb_face, DMC_AMBIGUOUS_FACE, sizeof(h.amb_face));
    memset(h.face_dir, 0, sizeof(h.face_dir));
    memcpy(h.face_dir, DMC_FACE_DIR, 6);
    for (int c = 0; c < 256; ++c) {
        uint16_t m = 0;
        for (int e = 0; e < 12; ++e)
            if (DMC_EDGE_LUT1[c * 12 + e] != 0xff) m |= (uint16_t)(1u << e);
        h.crossed[c] = m;
    }
}

dmc_status upload_tables(Ctx *ctx)
{
    DeviceTables h;
    fill_tables(h);
    CUDA_TRY(cudaMalloc(&ctx->d_tab, sizeof(DeviceTables)));
    CUDA_TRY(cudaMemcpy(ctx->d_tab, &h, sizeof(DeviceTables), cudaMemcpyHostToDevice));
    return DMC_OK;
}

struct OutBufs {
    void *v = nullptr, *q = nullptr, *t = nullptr;
    size_t vb = 0, qb = 0, tb = 0;
};

}  // namespace dmc

using namespace dmc;

struct dmc_ctx {
    Ctx c;
    OutBufs out;
};

namespace dmc {
Ctx *ctx_of(dmc_ctx *ctx) { return &ctx->c; }
}

static bool valid_volume(const dmc_volume *vol)
{
    if (!vol || !vol->data) return false;
    if (vol->dtype != DMC_F32 && vol->dtype != DMC_U16) return false;
    return true;
}

static dmc_status make_args(const dmc_volume *vol, const float mn[3], const float mx[3], float iso, ExtractArgs &a)
{
    if (!valid_volume(vol) || !mn || !mx) return DMC_ERR_INVALID_ARG;
    memset(&a, 0, sizeof(a));
    a.vol = vol->data;
    a.dtype = vol->dtype;
    a.pts = make_uint3(vol->dims[0], vol->dims[1], vol->dims[2]);
    uint3 c;
    c.x = vol->dims[0] > 0 ? vol->dims[0] - 1 : 0;
    c.y = vol->dims[1] > 0 ? vol->dims[1] - 1 : 0;
    c.z = vol->dims[2] > 0 ? vol->dims[2] - 1 : 0;
    a.cells = c;
    // 32-bit cell indices inside the kernels' per-axis math; the totals are 64-bit
    if (!cell_count(c, &a.n_cells) || a.n_cells >= (1ull << 40)) return DMC_ERR_UNSUPPORTED;
    a.iso = iso;
    a.mn = make_float3(mn[0], mn[1], mn[2]);
    // utils.hpp / dmc.cu:2149: xyz_range = xyz_max - xyz_min
    a.rng = make_float3(mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]);
    return DMC_OK;
}

static uint64_t volume_bytes(const dmc_volume *vol)
{
    return (uint64_t)vol->dims[0] * vol->dims[1] * vol->dims[2] * (vol->dtype == DMC_U16 ? 2 : 4);
}

// Runs the selected path.  On return *a.n_vertices/*a.n_quads hold the totals.
static dmc_status run_path(dmc_ctx *ctx, ExtractArgs &a, cudaStream_t st)
{
    Ctx *c = &ctx->c;
    int algo = c->algo;
    // smoothing needs per-cell offsets, which only the simple path keeps
    if (a.num_smooth && algo == DMC_ALGO_BRICK) return DMC_ERR_UNSUPPORTED;
    if (algo == DMC_ALGO_AUTO) algo = (brick_supports(a) && !a.num_smooth) ? DMC_ALGO_BRICK : DMC_ALGO_SIMPLE;
    if (algo == DMC_ALGO_BRICK && !brick_supports(a)) return DMC_ERR_UNSUPPORTED;
    c->stats.algo = algo;
    return algo == DMC_ALGO_BRICK ? brick_run(c, a, st) : simple_run(c, a, st);
}

static dmc_status finish(dmc_ctx *ctx, cudaStream_t st)
{
    Ctx *c = &ctx->c;
    CUDA_TRY(cudaEventRecord(c->ev1, st));
    CUDA_TRY(cudaMemcpyAsync(c->h_ctl, c->d_ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    event_ms(&c->stats.device_ms, c->ev0, c->ev1);
    if (c->evk_used >= 1) {
        event_ms(&c->stats.count_ms, c->evk[0], c->evk[1]);
        event_ms(&c->stats.scan_ms, c->evk[1], c->evk[2]);
    }
    if (c->evk_used >= 2) event_ms(&c->stats.emit_ms, c->evk[3], c->evk[4]);
    c->evk_used = 0;
    uint32_t err = c->h_ctl->err;
    if (err & DEV_ERR_TIMEOUT) return DMC_ERR_TIMEOUT;
    if (err & DEV_ERR_OVERFLOW) return DMC_ERR_OUTPUT_OVERFLOW;
    if (err & DEV_ERR_BOUNDS) return DMC_ERR_DEVICE_CHECK;
    return DMC_OK;
}

extern "C" {

const char *dmc_version(void) { return "gb300-dmc 0.1.0 (sm_103a)"; }

const char *dmc_tables_sha256(void) { return DMC_TABLES_SHA256; }

const char *dmc_last_cuda_error(void) { return g_last_cuda; }

const char *dmc_status_string(dmc_status s)
{
    switch (s) {
    case DMC_OK: return "ok";
    case DMC_ERR_INVALID_ARG: return "invalid argument";
    case DMC_ERR_OOM: return "out of device memory";
    case DMC_ERR_OUTPUT_OVERFLOW: return "output buffers too small or more than 2^32-1 vertices/quads";
    case DMC_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case DMC_ERR_CUDA: return "CUDA error";
    case DMC_ERR_UNSUPPORTED: return "unsupported input for the selected path";
    case DMC_ERR_DEVICE_CHECK: return "device-side bounds check failed";
    case DMC_ERR_TOO_LARGE: return "volume exceeds the fixed scratch of the no-allocation entry point";
    }
    return "unknown status";
}

dmc_status dmc_create(dmc_ctx **out, int device)
{
    if (!out) return DMC_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    const cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) set_last_cuda_error(e);
    if (e != cudaSuccess || device < 0 || device >= n) return DMC_ERR_INVALID_ARG;
    dmc_ctx *ctx = new (std::nothrow) dmc_ctx();
    if (!ctx) return DMC_ERR_OOM;
    Ctx *c = &ctx->c;
    c->device = device;
    dmc_status s = DMC_OK;
    do {
        if (cudaSetDevice(device) != cudaSuccess) { s = DMC_ERR_CUDA; break; }
        cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { s = DMC_ERR_CUDA; break; }
        if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) { s = DMC_ERR_CUDA; break; }
        for (int i = 0; i < 5; ++i)
            if (cudaEventCreate(&c->evk[i]) != cudaSuccess) { s = DMC_ERR_CUDA; break; }
        if (s != DMC_OK) break;
        if (cudaMalloc(&c->d_ctl, sizeof(DevCtl)) != cudaSuccess) { s = DMC_ERR_OOM; break; }
        if (cudaMallocHost(&c->h_ctl, sizeof(DevCtl)) != cudaSuccess) { s = DMC_ERR_OOM; break; }
        s = upload_tables(c);
    } while (0);
    if (s != DMC_OK) { dmc_destroy(ctx); return s; }
    *out = ctx;
    return DMC_OK;
}

dmc_status dmc_destroy(dmc_ctx *ctx)
{
    if (!ctx) return DMC_ERR_INVALID_ARG;
    Ctx *c = &ctx->c;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->scratch); cudaFree(c->d_ctl); cudaFree(c->d_tab); cudaFree(c->d_vol);
    cudaFree(ctx->out.v); cudaFree(ctx->out.q); cudaFree(ctx->out.t);
    if (c->h_ctl) cudaFreeHost(c->h_ctl);
    batch_state_free(c);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int i = 0; i < 5; ++i)
        if (c->evk[i]) cudaEventDestroy(c->evk[i]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete ctx;
    return DMC_OK;
}

dmc_status dmc_set_algo(dmc_ctx *ctx, dmc_algo algo)
{
    if (!ctx || algo < DMC_ALGO_AUTO || algo > DMC_ALGO_BRICK) return DMC_ERR_INVALID_ARG;
    ctx->c.algo = algo;
    return DMC_OK;
}

dmc_status dmc_get_stats(const dmc_ctx *ctx, dmc_stats *stats)
{
    if (!ctx || !stats) return DMC_ERR_INVALID_ARG;
    *stats = ctx->c.stats;
    return DMC_OK;
}

void dmc_mesh_free(dmc_mesh *m)
{
    if (!m) return;
    free(m->vertices); free(m->quads); free(m->triangles);
    memset(m, 0, sizeof(*m));
}

dmc_status dmc_extract_device(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                              float iso, uint32_t num_smooth, float *d_vertices, uint64_t vertex_capacity,
                              uint32_t *d_quads, uint64_t quad_capacity, uint32_t *d_triangles,
                              uint64_t *n_vertices, uint64_t *n_quads, void *stream)
{
    NvtxRange nvtx("dmc_extract_device");
    if (!ctx || !n_vertices || !n_quads) return DMC_ERR_INVALID_ARG;
    ExtractArgs a;
    dmc_status s = make_args(vol, xyz_min, xyz_max, iso, a);
    if (s != DMC_OK) return s;
    if ((vertex_capacity && !d_vertices) || (quad_capacity && !d_quads)) return DMC_ERR_INVALID_ARG;
    // smoothing walks the quad rings, so it needs the quad buffer with the vertices
    if (num_smooth && (!d_vertices) != (!d_quads)) return DMC_ERR_INVALID_ARG;
    a.num_smooth = num_smooth;
    Ctx *c = &ctx->c;
    if (c->batch_pending) return DMC_ERR_INVALID_ARG;   // an asynchronous batch holds the scratch
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    a.verts = d_vertices; a.vcap = vertex_capacity;
    a.quads = d_quads; a.qcap = quad_capacity;
    a.tris = d_triangles;
    a.n_vertices = n_vertices; a.n_quads = n_quads;
    a.sizing_only = !d_vertices && !d_quads && !d_triangles;
    *n_vertices = 0; *n_quads = 0;
    c->stats = dmc_stats{};
    CUDA_TRY(cudaEventRecord(c->ev0, st));
    if (a.n_cells == 0) return finish(ctx, st);
    s = run_path(ctx, a, st);
    dmc_status f = finish(ctx, st);
    if (s == DMC_OK) s = f;
    c->stats.n_vertices = *n_vertices;
    c->stats.n_quads = *n_quads;
    return s;
}

dmc_status dmc_extract_batch(dmc_ctx *ctx, const dmc_batch_item *items, uint32_t n_items, float *d_vertices,
                             uint64_t vertex_capacity, uint32_t *d_quads, uint64_t quad_capacity, uint32_t *d_triangles,
                             dmc_batch_result *d_results, dmc_batch_result *results, uint64_t *n_vertices,
                             uint64_t *n_quads, uint32_t flags, void *stream)
{
    NvtxRange nvtx("dmc_extract_batch");
    if (!ctx || !items || n_items == 0) return DMC_ERR_INVALID_ARG;
    if (flags & ~(DMC_BATCH_ASYNC | DMC_BATCH_GRAPH)) return DMC_ERR_INVALID_ARG;
    if ((vertex_capacity && !d_vertices) || (quad_capacity && !d_quads)) return DMC_ERR_INVALID_ARG;
    const bool async = flags != 0;
    if (!async && (!n_vertices || !n_quads)) return DMC_ERR_INVALID_ARG;
    Ctx *c = &ctx->c;
    if (c->batch_pending) return DMC_ERR_INVALID_ARG;   // dmc_batch_wait first
    std::vector<BrickItem> bi(n_items);
    for (uint32_t i = 0; i < n_items; ++i) {
        ExtractArgs a;
        dmc_status s = make_args(&items[i].vol, items[i].xyz_min, items[i].xyz_max, items[i].iso, a);
        if (s != DMC_OK) return s;
        BrickItem &it = bi[i];
        it.data = a.vol; it.dtype = a.dtype; it.pts = a.pts; it.cells = a.cells; it.iso = a.iso; it.mn = a.mn; it.rng = a.rng;
    }
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    BrickOut o{};
    o.verts = d_vertices; o.vcap = vertex_capacity;
    o.quads = d_quads; o.qcap = quad_capacity;
    o.tris = d_triangles;
    o.d_results = d_results;
    o.h_results = async ? nullptr : results;
    o.n_vertices = async ? nullptr : n_vertices;
    o.n_quads = async ? nullptr : n_quads;
    o.mode = (flags & DMC_BATCH_GRAPH) ? BATCH_GRAPH : async ? BATCH_ASYNC : BATCH_SYNC;
    o.sizing_only = !async && !d_vertices && !d_quads && !d_triangles;
    if (!async) { *n_vertices = 0; *n_quads = 0; }
    c->stats = dmc_stats{};
    c->stats.algo = DMC_ALGO_BRICK;
    c->evk_used = 0;
    CUDA_TRY(cudaEventRecord(c->ev0, st));
    dmc_status s = brick_extract(c, bi.data(), n_items, o, st);
    if (s != DMC_OK) return s;
    CUDA_TRY(cudaEventRecord(c->ev1, st));
    if (async) {
        c->batch_pending = true;
        return DMC_OK;
    }
    cudaEventSynchronize(c->ev1);
    event_ms(&c->stats.device_ms, c->ev0, c->ev1);
    if (c->evk_used >= 2) {
        event_ms(&c->stats.count_ms, c->evk[0], c->evk[1]);
        event_ms(&c->stats.scan_ms, c->evk[1], c->evk[2]);
        event_ms(&c->stats.emit_ms, c->evk[3], c->evk[4]);
    }
    c->evk_used = 0;
    return DMC_OK;
}

dmc_status dmc_batch_wait(dmc_ctx *ctx, dmc_batch_result *results, uint64_t *n_vertices, uint64_t *n_quads)
{
    NvtxRange nvtx("dmc_batch_wait");
    if (!ctx) return DMC_ERR_INVALID_ARG;
    Ctx *c = &ctx->c;
    if (!c->batch_pending) return DMC_ERR_INVALID_ARG;
    c->batch_pending = false;
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    dmc_status s = brick_wait(c, results, n_vertices, n_quads);
    event_ms(&c->stats.device_ms, c->ev0, c->ev1);
    return s;
}

dmc_status dmc_shard_count(dmc_ctx *ctx, const dmc_volume *local, uint32_t nz, uint32_t z_begin, uint32_t z_end,
                           const float xyz_min[3], const float xyz_max[3], float iso,
                           uint64_t *n_vertices, uint64_t *n_quads, void *stream)
{
    NvtxRange nvtx("dmc_shard_count");
    if (!ctx || !local || !n_vertices || !n_quads) return DMC_ERR_INVALID_ARG;
    *n_vertices = 0; *n_quads = 0;
    if (nz < 2 || z_begin >= z_end || z_end > nz - 1) return DMC_ERR_INVALID_ARG;
    const uint32_t p0 = z_begin > 0 ? z_begin - 1 : 0, p1 = std::min<uint32_t>(z_end + 3, nz);
    if (local->dims[2] != p1 - p0) return DMC_ERR_INVALID_ARG;
    dmc_volume whole = *local;
    whole.dims[2] = nz;
    ExtractArgs a;
    dmc_status s = make_args(&whole, xyz_min, xyz_max, iso, a);
    if (s != DMC_OK) return s;
    if (!brick_supports(a)) return DMC_ERR_UNSUPPORTED;
    Ctx *c = &ctx->c;
    if (c->batch_pending) return DMC_ERR_INVALID_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    BrickItem it;
    it.data = local->data; it.dtype = local->dtype; it.pts = a.pts; it.cells = a.cells; it.iso = a.iso;
    it.mn = a.mn; it.rng = a.rng;
    c->stats = dmc_stats{};
    c->stats.algo = DMC_ALGO_BRICK;
    s = brick_shard_count(c, it, p0, z_begin, z_end, n_vertices, n_quads, st);
    event_ms(&c->stats.device_ms, c->ev0, c->ev1);
    return s;
}

dmc_status dmc_shard_emit(dmc_ctx *ctx, uint64_t vertex_offset, float *d_vertices, uint64_t vertex_capacity,
                          uint32_t *d_quads, uint64_t quad_capacity, uint32_t *d_triangles, void *stream)
{
    NvtxRange nvtx("dmc_shard_emit");
    if (!ctx) return DMC_ERR_INVALID_ARG;
    if ((vertex_capacity && !d_vertices) || (quad_capacity && !d_quads)) return DMC_ERR_INVALID_ARG;
    Ctx *c = &ctx->c;
    if (c->batch_pending) return DMC_ERR_INVALID_ARG;
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    BrickOut o{};
    o.verts = d_vertices; o.vcap = vertex_capacity; o.quads = d_quads; o.qcap = quad_capacity; o.tris = d_triangles;
    dmc_status s = brick_shard_emit(c, vertex_offset, o, st);
    if (s == DMC_OK) event_ms(&c->stats.emit_ms, c->ev0, c->ev1);
    return s;
}

dmc_status dmc_set_option(dmc_ctx *ctx, dmc_option opt, int64_t value)
{
    if (!ctx) return DMC_ERR_INVALID_ARG;
    switch (opt) {
    case DMC_OPT_BRICK_PLANES:
        if (value < 0 || value > 256) return DMC_ERR_INVALID_ARG;
        ctx->c.brick_zc = (uint32_t)value;
        return DMC_OK;
    case DMC_OPT_STREAM_SLABS:
        if (value < 0 || value > 32) return DMC_ERR_INVALID_ARG;
        ctx->c.stream_slabs = (uint32_t)value;
        return DMC_OK;
    case DMC_OPT_FAIL_ALLOCS:
        if (value < 0 || value > 1000) return DMC_ERR_INVALID_ARG;
        ctx->c.fail_allocs = (uint32_t)value;
        return DMC_OK;
    }
    return DMC_ERR_INVALID_ARG;
}

// Host-volume extraction into the context's device output buffers (grown
// as needed); the totals come back in *V, *Q.
static dmc_status run_host(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                           float iso, uint32_t num_smooth, int want_triangles, uint64_t *V, uint64_t *Q)
{
    ExtractArgs a;
    dmc_status s = make_args(vol, xyz_min, xyz_max, iso, a);
    if (s != DMC_OK) return s;
    a.num_smooth = num_smooth;
    Ctx *c = &ctx->c;
    if (c->batch_pending) return DMC_ERR_INVALID_ARG;   // an asynchronous batch holds the scratch
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    cudaStream_t st = c->stream;
    c->stats = dmc_stats{};
    *V = 0; *Q = 0;
    a.n_vertices = V; a.n_quads = Q;
    CUDA_TRY(cudaEventRecord(c->ev0, st));
    if (a.n_cells > 0) {
        // upload the host volume (dmc.cu:2077-2079)
        uint64_t bytes = volume_bytes(vol);
        s = reserve(c, &c->d_vol, &c->d_vol_bytes, bytes);
        if (s != DMC_OK) return s;
        CUDA_TRY(cudaMemcpyAsync(c->d_vol, vol->data, bytes, cudaMemcpyHostToDevice, st));
        a.vol = c->d_vol;
        // first try into the context's output buffers as they are; grow and
        // retry once if the mesh is larger
        for (int attempt = 0; attempt < 2; ++attempt) {
            a.verts = (float *)ctx->out.v; a.vcap = ctx->out.vb / 12;
            a.quads = (uint32_t *)ctx->out.q; a.qcap = ctx->out.qb / 16;
            a.tris = want_triangles ? (uint32_t *)ctx->out.t : nullptr;
            if (want_triangles && ctx->out.tb / 24 < a.qcap) a.qcap = ctx->out.tb / 24;
            s = run_path(ctx, a, st);
            if (s != DMC_ERR_OUTPUT_OVERFLOW || attempt == 1) break;
            if (*V >= 0xFFFFFFFFull || *Q >= 0xFFFFFFFFull) break;
            if ((s = reserve(c, &ctx->out.v, &ctx->out.vb, 12 * (*V ? *V : 1))) != DMC_OK) return s;
            if ((s = reserve(c, &ctx->out.q, &ctx->out.qb, 16 * (*Q ? *Q : 1))) != DMC_OK) return s;
            if (want_triangles && (s = reserve(c, &ctx->out.t, &ctx->out.tb, 24 * (*Q ? *Q : 1))) != DMC_OK) return s;
            CUDA_TRY(cudaMemsetAsync(c->d_ctl, 0, sizeof(DevCtl), st));
        }
        if (s != DMC_OK) { finish(ctx, st); return s; }
    }
    s = finish(ctx, st);
    c->stats.n_vertices = *V; c->stats.n_quads = *Q;
    return s;
}

// internal status of run_streamed: the streamed path does not apply
constexpr dmc_status kNotStreamed = (dmc_status)-1;

// Streamed dmc_run_into (brick path, no smoothing): the volume goes up in z
// slabs while earlier slabs are extracted and their meshes come down.  Taken
// for volumes of 64 MiB and more unless the option says otherwise; returns
// kNotStreamed when it does not apply.
static dmc_status run_streamed(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                               float iso, uint32_t num_smooth, float *hv, uint64_t vcap, uint32_t *hq, uint64_t qcap,
                               uint32_t *ht, uint64_t *V, uint64_t *Q, bool *dev_short)
{
    Ctx *c = &ctx->c;
    *dev_short = false;
    if (c->stream_slabs == 1 || num_smooth || c->algo == DMC_ALGO_SIMPLE || c->batch_pending) return kNotStreamed;
    ExtractArgs a;
    dmc_status s = make_args(vol, xyz_min, xyz_max, iso, a);
    if (s != DMC_OK || a.n_cells == 0 || !brick_supports(a)) return kNotStreamed;
    const uint64_t bytes = volume_bytes(vol);
    uint32_t slabs = c->stream_slabs;
    if (slabs == 0) {
        if (bytes < (64ull << 20)) return kNotStreamed;
        slabs = (uint32_t)std::min<uint64_t>(32, std::max<uint64_t>(2, bytes / (96ull << 20)));   // 21 at 2 GiB
    }
    // the context's device output buffers as they are: too small ones make
    // the caller take the plain path, which grows them
    if (!ctx->out.v || !ctx->out.q || (ht && !ctx->out.t)) { *dev_short = true; return DMC_ERR_OUTPUT_OVERFLOW; }
    if (cudaSetDevice(c->device) != cudaSuccess) return DMC_ERR_CUDA;
    if ((s = reserve(c, &c->d_vol, &c->d_vol_bytes, bytes)) != DMC_OK) return s;
    c->stats = dmc_stats{};
    c->stats.algo = DMC_ALGO_BRICK;
    a.vol = c->d_vol;
    a.verts = (float *)ctx->out.v; a.vcap = ctx->out.vb / 12;
    a.quads = (uint32_t *)ctx->out.q; a.qcap = ctx->out.qb / 16;
    a.tris = ht ? (uint32_t *)ctx->out.t : nullptr;
    if (ht && ctx->out.tb / 24 < a.qcap) a.qcap = ctx->out.tb / 24;
    StreamIO io{vol->data, hv, vcap, hq, qcap, ht};
    s = brick_run_streamed(c, a, io, slabs, dev_short, c->stream);
    *V = c->stats.n_vertices; *Q = c->stats.n_quads;
    return s;
}

// download the mesh (dmc.cu:2197-2205) from the context's device buffers
static dmc_status download(dmc_ctx *ctx, uint64_t V, uint64_t Q, float *hv, uint32_t *hq, uint32_t *ht)
{
    cudaStream_t st = ctx->c.stream;
    if (V) CUDA_TRY(cudaMemcpyAsync(hv, ctx->out.v, 12 * V, cudaMemcpyDeviceToHost, st));
    if (Q && hq) CUDA_TRY(cudaMemcpyAsync(hq, ctx->out.q, 16 * Q, cudaMemcpyDeviceToHost, st));
    if (Q && ht) CUDA_TRY(cudaMemcpyAsync(ht, ctx->out.t, 24 * Q, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return DMC_OK;
}

// Write one byte per page of freshly allocated host buffers, from several
// threads.  The pages of a large malloc are mapped on first touch; taking
// those faults in parallel here is many times faster than taking them one at
// a time inside the device-to-host copy (or the driver's staging copy).
static void touch_pages(void *const *bufs, const uint64_t *bytes, int n)
{
    const long ps = sysconf(_SC_PAGESIZE);
    const uint64_t page = ps > 0 ? (uint64_t)ps : 4096;
    uint64_t total = 0;
    for (int i = 0; i < n; ++i) total += bytes[i];
    unsigned nt = std::thread::hardware_concurrency();
    nt = std::min<unsigned>(nt ? nt : 1, 32);
    if (total < (32ull << 20) || nt < 2) return;   // small meshes: the copy takes the faults
    const uint64_t share = (total / nt + page - 1) / page * page;
    auto work = [=](uint64_t lo, uint64_t hi) {
        uint64_t base = 0;
        for (int i = 0; i < n; ++i) {
            const uint64_t b0 = std::max(lo, base), b1 = std::min(hi, base + bytes[i]);
            for (uint64_t o = b0; o < b1; o += page) ((volatile char *)bufs[i])[o - base] = 0;
            base += bytes[i];
        }
    };
    std::vector<std::thread> th;
    try {
        for (unsigned k = 1; k < nt && k * share < total; ++k)
            th.emplace_back(work, k * share, std::min(total, (k + 1) * share));
    } catch (...) {
        // no more threads: the ones started and this one cover what they can
    }
    work(0, std::min(total, share));
    for (auto &t : th) t.join();
}

dmc_status dmc_run(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                   float iso, uint32_t num_smooth, int want_triangles, dmc_mesh *out)
{
    NvtxRange nvtx("dmc_run");
    if (!ctx || !out) return DMC_ERR_INVALID_ARG;
    memset(out, 0, sizeof(*out));
    uint64_t V = 0, Q = 0;
    dmc_status s = run_host(ctx, vol, xyz_min, xyz_max, iso, num_smooth, want_triangles, &V, &Q);
    if (s != DMC_OK) return s;
    out->n_vertices = V; out->n_quads = Q; out->n_triangles = want_triangles ? 2 * Q : 0;
    out->vertices = (float *)malloc(V ? 12 * V : 1);
    out->quads = (uint32_t *)malloc(Q ? 16 * Q : 1);
    if (want_triangles) out->triangles = (uint32_t *)malloc(Q ? 24 * Q : 1);
    if (!out->vertices || !out->quads || (want_triangles && !out->triangles)) { dmc_mesh_free(out); return DMC_ERR_OOM; }
    void *bufs[3] = {out->vertices, out->quads, out->triangles};
    const uint64_t sizes[3] = {12 * V, 16 * Q, want_triangles ? 24 * Q : 0};
    touch_pages(bufs, sizes, 3);
    return download(ctx, V, Q, out->vertices, out->quads, want_triangles ? out->triangles : nullptr);
}

dmc_status dmc_run_into(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                        float iso, uint32_t num_smooth, float *h_vertices, uint64_t vertex_capacity,
                        uint32_t *h_quads, uint64_t quad_capacity, uint32_t *h_triangles,
                        uint64_t *n_vertices, uint64_t *n_quads)
{
    NvtxRange nvtx("dmc_run_into");
    if (!ctx || !n_vertices || !n_quads) return DMC_ERR_INVALID_ARG;
    if ((vertex_capacity && !h_vertices) || (quad_capacity && !h_quads && !h_triangles)) return DMC_ERR_INVALID_ARG;
    *n_vertices = 0; *n_quads = 0;
    uint64_t V = 0, Q = 0;
    bool dev_short = false;
    dmc_status s = run_streamed(ctx, vol, xyz_min, xyz_max, iso, num_smooth, h_vertices, vertex_capacity, h_quads,
                                quad_capacity, h_triangles, &V, &Q, &dev_short);
    if (s != kNotStreamed && !(s == DMC_ERR_OUTPUT_OVERFLOW && dev_short)) {
        *n_vertices = V; *n_quads = Q;
        return s;
    }
    // not streamed, or the context's device buffers were too small: the
    // plain path grows them (and they stay for the next call)
    s = run_host(ctx, vol, xyz_min, xyz_max, iso, num_smooth, h_triangles != nullptr, &V, &Q);
    *n_vertices = V; *n_quads = Q;
    if (s != DMC_OK) return s;
    if (V > vertex_capacity || Q > quad_capacity) return DMC_ERR_OUTPUT_OVERFLOW;
    return download(ctx, V, Q, h_vertices, h_quads, h_triangles);
}

}  // extern "C"
