// Serving loop: a device-resident pool of volumes, (volume, isovalue)
// requests admitted by a worst-case output bound, and continuous batching of
// the admitted requests onto a few lanes, each a context with its own stream
// and captured batch graph, so that batches overlap on the device.
//
// A request's worst-case output is 7 vertices and 3 quads per cell: at most
// 4 dual vertices plus one crossing on each of the 3 edges a cell owns, and
// one quad per owned edge (dmc.cu:1382-1406, 1983-2008).  A batch takes one
// slice of the vertex arena and one of the quad arena sized by the sum of
// its requests' bounds; when it completes, each slice shrinks to the mesh
// actually written, and it returns to the arena when every request of the
// batch has been released.
//
// One scheduler thread owns the lanes.  Per iteration it (1) completes lanes
// whose batch event has fired, (2) fills idle lanes from the FIFO of pending
// requests while their bounds fit the arenas, and (3) sleeps until a submit,
// a release or, with lanes busy, a short poll interval.  Requests that arrive
// while other batches run join the next batch as soon as a lane and arena
// space are free.
#include <stdint.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <list>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/dmc_gb300.h"
#include "dmc_arena.h"
#include "dmc_internal.h"   // NvtxRange

namespace {

using Clock = std::chrono::steady_clock;
constexpr uint64_t kVertsPerCell = 7, kQuadsPerCell = 3;

struct PoolVolume {
    dmc_volume vol;
    float mn[3], mx[3];
    uint64_t cells;
};

struct Batch;

struct Request {
    uint64_t id = 0;
    uint32_t volume = 0;
    float iso = 0.f;
    uint64_t vbound = 0, qbound = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    bool done = false, released = false;
    dmc_status status = DMC_OK;
    uint64_t n_vertices = 0, n_quads = 0;
    uint64_t v_off = 0, q_off = 0;      // element offsets in the arenas
    uint32_t batch_size = 0;
    Batch *batch = nullptr;
};

struct Batch {
    uint64_t v_off = 0, v_len = 0, q_off = 0, q_len = 0;
    uint32_t live = 0;                   // requests not yet released
    bool complete = false;
};

struct Lane {
    dmc_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev = nullptr;
    bool busy = false;
    Batch *batch = nullptr;
    std::vector<Request *> reqs;
    std::vector<dmc_batch_item> items;
    std::vector<dmc_batch_result> res;
};

}  // namespace

struct dmc_server {
    dmc_server_config cfg{};
    Clock::time_point t0;
    float *verts = nullptr;
    uint32_t *quads = nullptr, *tris = nullptr;
    dmc::Arena va, qa;
    std::vector<PoolVolume> pool;
    std::vector<Lane> lanes;
    std::list<std::unique_ptr<Batch>> batches;
    std::unordered_map<uint64_t, Request> reqs;
    std::deque<Request *> pending;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::thread loop;
    bool stopping = false;
    uint64_t next_id = 1;
    dmc_server_stats stats{};

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
    bool launch(Lane &L, std::unique_lock<std::mutex> &lk);
    void complete(Lane &L, std::unique_lock<std::mutex> &lk);
    void free_batch(Batch *b);
};

void dmc_server::free_batch(Batch *b)
{
    va.release(b->v_off, b->v_len);
    qa.release(b->q_off, b->q_len);
    batches.remove_if([b](const std::unique_ptr<Batch> &p) { return p.get() == b; });
}

// Forms a batch from the head of the FIFO and launches it on lane L.
bool dmc_server::launch(Lane &L, std::unique_lock<std::mutex> &lk)
{
    dmc::NvtxRange nvtx("dmc_server batch launch");
    const uint32_t maxb = cfg.plain ? 1u : cfg.max_batch;
    const uint64_t vfree = va.largest_free(), qfree = qa.largest_free();
    uint64_t vsum = 0, qsum = 0;
    L.reqs.clear();
    while (!pending.empty() && L.reqs.size() < maxb) {
        Request *r = pending.front();
        const uint64_t v2 = vsum + dmc::Arena::round(r->vbound), q2 = qsum + dmc::Arena::round(r->qbound);
        if (v2 > vfree || q2 > qfree) break;
        vsum = v2; qsum = q2;
        L.reqs.push_back(r);
        pending.pop_front();
    }
    if (L.reqs.empty()) return false;
    auto b = std::make_unique<Batch>();
    b->v_off = va.alloc(vsum);
    b->q_off = qa.alloc(qsum);
    b->v_len = vsum; b->q_len = qsum;
    b->live = (uint32_t)L.reqs.size();
    L.batch = b.get();
    batches.push_back(std::move(b));
    const double t = now();
    L.items.resize(L.reqs.size());
    L.res.resize(L.reqs.size());
    for (size_t i = 0; i < L.reqs.size(); ++i) {
        Request *r = L.reqs[i];
        r->t_start = t;
        r->batch = L.batch;
        r->batch_size = (uint32_t)L.reqs.size();
        const PoolVolume &pv = pool[r->volume];
        L.items[i].vol = pv.vol;
        L.items[i].iso = r->iso;
        memcpy(L.items[i].xyz_min, pv.mn, sizeof(pv.mn));
        memcpy(L.items[i].xyz_max, pv.mx, sizeof(pv.mx));
    }
    L.busy = true;
    stats.batches++;
    if (L.reqs.size() > stats.max_batch_seen) stats.max_batch_seen = L.reqs.size();
    stats.arena_peak_vertices = va.peak();
    stats.arena_peak_quads = qa.peak();
    float *v = verts + 3 * L.batch->v_off;
    uint32_t *q = quads + 4 * L.batch->q_off;
    uint32_t *tr = tris ? tris + 6 * L.batch->q_off : nullptr;
    const uint64_t vcap = L.batch->v_len, qcap = L.batch->q_len;
    lk.unlock();
    dmc_status s;
    if (cfg.plain) {
        // the plain form: one synchronous extraction per request
        uint64_t nv = 0, nq = 0;
        const dmc_batch_item &it = L.items[0];
        s = dmc_extract_device(L.ctx, &it.vol, it.xyz_min, it.xyz_max, it.iso, 0, v, vcap, q, qcap, tr, &nv, &nq,
                               L.stream);
        L.res[0] = dmc_batch_result{0, nv, 0, nq};
    } else {
        s = dmc_extract_batch(L.ctx, L.items.data(), (uint32_t)L.items.size(), v, vcap, q, qcap, tr, nullptr,
                              nullptr, nullptr, nullptr, DMC_BATCH_GRAPH, L.stream);
    }
    if (s == DMC_OK && cudaEventRecord(L.ev, L.stream) != cudaSuccess) s = DMC_ERR_CUDA;
    lk.lock();
    if (s != DMC_OK) {
        // nothing is in flight: fail the batch's requests now
        for (Request *r : L.reqs) { r->status = s; r->done = true; r->t_done = now(); }
        L.batch->complete = true;
        L.busy = false;
        stats.completed += L.reqs.size();
        cv_done.notify_all();
    }
    return true;
}

void dmc_server::complete(Lane &L, std::unique_lock<std::mutex> &lk)
{
    dmc::NvtxRange nvtx("dmc_server batch complete");
    uint64_t V = 0, Q = 0;
    dmc_status s = DMC_OK;
    lk.unlock();
    if (!cfg.plain) s = dmc_batch_wait(L.ctx, L.res.data(), &V, &Q);
    else { V = L.res[0].n_vertices; Q = L.res[0].n_quads; }
    lk.lock();
    const double t = now();
    Batch *b = L.batch;
    for (size_t i = 0; i < L.reqs.size(); ++i) {
        Request *r = L.reqs[i];
        r->status = s;
        r->n_vertices = L.res[i].n_vertices;
        r->n_quads = L.res[i].n_quads;
        r->v_off = b->v_off + L.res[i].vertex_offset;
        r->q_off = b->q_off + L.res[i].quad_offset;
        r->t_done = t;
        r->done = true;
    }
    // keep only what was written
    if (s == DMC_OK) {
        b->v_len = va.shrink(b->v_off, b->v_len, V);
        b->q_len = qa.shrink(b->q_off, b->q_len, Q);
    }
    b->complete = true;
    if (b->live == 0) free_batch(b);
    stats.completed += L.reqs.size();
    L.busy = false;
    L.batch = nullptr;
    cv_done.notify_all();
}

void dmc_server::run()
{
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        bool any_busy = false;
        for (Lane &L : lanes) any_busy |= L.busy;
        if (stopping && !any_busy) break;
        bool progress = false;
        for (Lane &L : lanes) {
            if (!L.busy) continue;
            lk.unlock();
            const cudaError_t q = cudaEventQuery(L.ev);
            lk.lock();
            if (q == cudaSuccess) { complete(L, lk); progress = true; }
            else if (q != cudaErrorNotReady) {
                // the lane's work failed: report it on its requests
                for (Request *r : L.reqs) { r->status = DMC_ERR_CUDA; r->done = true; r->t_done = now(); }
                L.batch->complete = true;
                if (L.batch->live == 0) free_batch(L.batch);
                stats.completed += L.reqs.size();
                L.busy = false;
                cv_done.notify_all();
                progress = true;
            }
        }
        if (!stopping) {
            for (Lane &L : lanes) {
                if (L.busy || pending.empty()) continue;
                if (launch(L, lk)) progress = true;
                else break;                      // the head request waits for arena space
            }
        }
        if (progress) continue;
        any_busy = false;
        for (Lane &L : lanes) any_busy |= L.busy;
        if (any_busy) cv_sched.wait_for(lk, std::chrono::microseconds(20));
        else if (!stopping) cv_sched.wait_for(lk, std::chrono::milliseconds(50));
    }
}

extern "C" {

dmc_status dmc_server_create(const dmc_server_config *cfg, dmc_server **out)
{
    if (!cfg || !out) return DMC_ERR_INVALID_ARG;
    *out = nullptr;
    if (cfg->vertex_arena == 0 || cfg->quad_arena == 0) return DMC_ERR_INVALID_ARG;
    if (cfg->vertex_arena >= (1ull << 32) || cfg->quad_arena >= (1ull << 32)) return DMC_ERR_UNSUPPORTED;
    std::unique_ptr<dmc_server> s(new (std::nothrow) dmc_server());
    if (!s) return DMC_ERR_OOM;
    s->cfg = *cfg;
    if (!s->cfg.lanes) s->cfg.lanes = 2;
    if (!s->cfg.max_batch) s->cfg.max_batch = 64;
    if (s->cfg.plain) s->cfg.lanes = 1;
    s->t0 = Clock::now();
    if (cudaSetDevice(cfg->device) != cudaSuccess) return DMC_ERR_INVALID_ARG;
    auto fail = [&](dmc_status st) {
        for (Lane &L : s->lanes) {
            if (L.ev) cudaEventDestroy(L.ev);
            if (L.stream) cudaStreamDestroy(L.stream);
            if (L.ctx) dmc_destroy(L.ctx);
        }
        cudaFree(s->verts); cudaFree(s->quads); cudaFree(s->tris);
        return st;
    };
    const uint64_t vcap = dmc::Arena::round(cfg->vertex_arena), qcap = dmc::Arena::round(cfg->quad_arena);
    if (cudaMalloc(&s->verts, 12 * vcap) != cudaSuccess) return fail(DMC_ERR_OOM);
    if (cudaMalloc(&s->quads, 16 * qcap) != cudaSuccess) return fail(DMC_ERR_OOM);
    if (cfg->want_triangles && cudaMalloc(&s->tris, 24 * qcap) != cudaSuccess) return fail(DMC_ERR_OOM);
    s->va.reset(vcap);
    s->qa.reset(qcap);
    s->lanes.resize(s->cfg.lanes);
    for (Lane &L : s->lanes) {
        dmc_status st = dmc_create(&L.ctx, cfg->device);
        if (st != DMC_OK) return fail(st);
        if (cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking) != cudaSuccess) return fail(DMC_ERR_CUDA);
        if (cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming) != cudaSuccess) return fail(DMC_ERR_CUDA);
    }
    dmc_server *p = s.release();
    p->loop = std::thread([p] {
        cudaSetDevice(p->cfg.device);
        p->run();
    });
    *out = p;
    return DMC_OK;
}

dmc_status dmc_server_destroy(dmc_server *s)
{
    if (!s) return DMC_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        // requests never admitted fail; batches in flight complete first
        for (Request *r : s->pending) { r->status = DMC_ERR_INVALID_ARG; r->done = true; }
        s->pending.clear();
    }
    s->cv_sched.notify_all();
    s->cv_done.notify_all();
    if (s->loop.joinable()) s->loop.join();
    cudaSetDevice(s->cfg.device);
    for (Lane &L : s->lanes) {
        if (L.stream) cudaStreamSynchronize(L.stream);
        if (L.ev) cudaEventDestroy(L.ev);
        if (L.stream) cudaStreamDestroy(L.stream);
        if (L.ctx) dmc_destroy(L.ctx);
    }
    cudaFree(s->verts); cudaFree(s->quads); cudaFree(s->tris);
    delete s;
    return DMC_OK;
}

dmc_status dmc_server_add_volume(dmc_server *s, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                                 uint32_t *volume_id)
{
    if (!s || !vol || !vol->data || !xyz_min || !xyz_max || !volume_id) return DMC_ERR_INVALID_ARG;
    if (vol->dtype != DMC_F32 && vol->dtype != DMC_U16) return DMC_ERR_INVALID_ARG;
    PoolVolume pv;
    pv.vol = *vol;
    memcpy(pv.mn, xyz_min, sizeof(pv.mn));
    memcpy(pv.mx, xyz_max, sizeof(pv.mx));
    uint64_t c[3];
    for (int k = 0; k < 3; ++k) c[k] = vol->dims[k] ? vol->dims[k] - 1 : 0;
    pv.cells = c[0] * c[1] * c[2];
    std::lock_guard<std::mutex> lk(s->mu);
    if (pv.cells * kVertsPerCell > s->va.capacity() || pv.cells * kQuadsPerCell > s->qa.capacity())
        return DMC_ERR_OUTPUT_OVERFLOW;   // could never be admitted
    *volume_id = (uint32_t)s->pool.size();
    s->pool.push_back(pv);
    return DMC_OK;
}

dmc_status dmc_server_submit(dmc_server *s, uint32_t volume_id, float iso, uint64_t *request_id)
{
    if (!s || !request_id) return DMC_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stopping || volume_id >= s->pool.size()) return DMC_ERR_INVALID_ARG;
        const uint64_t id = s->next_id++;
        Request &r = s->reqs[id];
        r.id = id;
        r.volume = volume_id;
        r.iso = iso;
        r.vbound = s->pool[volume_id].cells * kVertsPerCell;
        r.qbound = s->pool[volume_id].cells * kQuadsPerCell;
        r.t_submit = s->now();
        s->pending.push_back(&r);
        s->stats.submitted++;
        *request_id = id;
    }
    s->cv_sched.notify_one();
    return DMC_OK;
}

dmc_status dmc_server_wait(dmc_server *s, uint64_t request_id, double timeout_s, dmc_server_result *out)
{
    if (!s || !out) return DMC_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(request_id);
    if (it == s->reqs.end() || it->second.released) return DMC_ERR_INVALID_ARG;
    Request &r = it->second;
    if (!r.done) {
        const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                              std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0.0));
        s->cv_done.wait_until(lk, until, [&] { return r.done; });
        if (!r.done) return DMC_ERR_TIMEOUT;
    }
    memset(out, 0, sizeof(*out));
    out->status = r.status;
    out->n_vertices = r.n_vertices;
    out->n_quads = r.n_quads;
    if (r.status == DMC_OK) {
        out->vertices = s->verts + 3 * r.v_off;
        out->quads = s->quads + 4 * r.q_off;
        out->triangles = s->tris ? s->tris + 6 * r.q_off : nullptr;
    }
    out->t_submit = r.t_submit;
    out->t_start = r.t_start;
    out->t_done = r.t_done;
    out->batch_size = r.batch_size;
    return DMC_OK;
}

dmc_status dmc_server_release(dmc_server *s, uint64_t request_id)
{
    if (!s) return DMC_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->reqs.find(request_id);
        if (it == s->reqs.end() || !it->second.done) return DMC_ERR_INVALID_ARG;
        Batch *b = it->second.batch;
        s->reqs.erase(it);
        if (b && --b->live == 0 && b->complete) s->free_batch(b);
    }
    s->cv_sched.notify_one();
    return DMC_OK;
}

dmc_status dmc_server_get_stats(dmc_server *s, dmc_server_stats *out)
{
    if (!s || !out) return DMC_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->arena_peak_vertices = s->va.peak();
    out->arena_peak_quads = s->qa.peak();
    return DMC_OK;
}

dmc_status dmc_server_replay(dmc_server *s, uint32_t n, const uint32_t *volume_ids, const float *isos,
                             const double *arrival_s, double *latency_s, dmc_status *status)
{
    if (!s || (n && (!volume_ids || !isos || !arrival_s || !latency_s || !status))) return DMC_ERR_INVALID_ARG;
    std::vector<uint64_t> ids(n, 0);
    std::vector<dmc_status> sub(n, DMC_OK);
    std::atomic<uint32_t> submitted{0};
    const Clock::time_point start = Clock::now();
    std::thread producer([&] {
        for (uint32_t i = 0; i < n; ++i) {
            const auto due = start + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
            if (due - Clock::now() > std::chrono::microseconds(200)) std::this_thread::sleep_until(due - std::chrono::microseconds(100));
            while (Clock::now() < due) { }
            sub[i] = dmc_server_submit(s, volume_ids[i], isos[i], &ids[i]);
            submitted.store(i + 1, std::memory_order_release);
        }
    });
    for (uint32_t i = 0; i < n; ++i) {
        while (submitted.load(std::memory_order_acquire) <= i) std::this_thread::yield();
        if (sub[i] != DMC_OK) { status[i] = sub[i]; latency_s[i] = -1.0; continue; }
        dmc_server_result r;
        dmc_status w = dmc_server_wait(s, ids[i], 3600.0, &r);
        status[i] = w != DMC_OK ? w : r.status;
        latency_s[i] = w == DMC_OK ? r.t_done - r.t_submit : -1.0;
        dmc_server_release(s, ids[i]);
    }
    producer.join();
    return DMC_OK;
}

}  // extern "C"
