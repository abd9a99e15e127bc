/*
 * dmc_gb300.h — C ABI of the GB300 Dual Marching Cubes extractor.
 *
 * The reference (vcg-thin-meshgen/Framework, DMC_CUDA/DMC_CUDA/include/dmc.hpp)
 * exposes three C++ calls: dmc::setup_device_luts() (dmc.hpp:40),
 * dmc::run_dmc(vertices, triangles, grid, xyz_min, xyz_max, iso, num_smooth)
 * (dmc.hpp:56-57) and dmc::cleanup_device_luts() (dmc.hpp:48).  Each entry
 * point below names the reference call it replaces.  The ABI uses only plain
 * pointers, sizes and enums, so any FFI (ctypes, cgo, JNI, N-API) can bind it.
 *
 * Conventions
 *  - Volumes are x-fastest: sample (x, y, z) is data[(z * ny + y) * nx + x]
 *    (utils::Array3D, utils.hpp:38).  dims are point counts; the cell grid is
 *    (nx-1) x (ny-1) x (nz-1).
 *  - World coordinates follow utils::ijk_to_xyz (utils.hpp:118-122):
 *    x(i) = (float)i / (nx-1) * (xyz_max.x - xyz_min.x) + xyz_min.x.
 *  - Output order matches the reference: vertices grouped by active cell in
 *    ascending cell index, dual vertices first, then the crossings of the
 *    cell's own edges 6, 9, 10; quads grouped by owner cell, edges 6, 9, 10.
 *    Triangles are the reference's split (q0,q1,q2), (q2,q3,q0).
 *  - Errors are returned as dmc_status; nothing prints or exits (the reference
 *    calls exit(1) on any CUDA error, cuda_includes.h:13-19).
 *  - A context is used by one host thread at a time; use one context per
 *    thread.  Calls on different contexts may run concurrently.
 */
#ifndef DMC_GB300_H
#define DMC_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    DMC_OK = 0,
    DMC_ERR_INVALID_ARG = 1,
    DMC_ERR_OOM = 2,
    DMC_ERR_OUTPUT_OVERFLOW = 3,   /* caller buffers too small, or > 2^32-1 vertices/quads */
    DMC_ERR_TIMEOUT = 4,           /* a bounded device-side wait gave up */
    DMC_ERR_CUDA = 5,
    DMC_ERR_UNSUPPORTED = 6,
    DMC_ERR_DEVICE_CHECK = 7,      /* a device-side bounds check failed */
    DMC_ERR_TOO_LARGE = 8          /* volume exceeds the fixed scratch of dmc_extract_device_noalloc */
} dmc_status;

typedef enum { DMC_F32 = 0, DMC_U16 = 1 } dmc_dtype;

/* kernel family used by an extraction */
typedef enum {
    DMC_ALGO_AUTO = 0,      /* the fastest path for the input */
    DMC_ALGO_SIMPLE = 1,    /* per-cell arrays + look-back scan (cross-check path) */
    DMC_ALGO_BRICK = 2      /* bit-sliced brick sweep, count/scan/emit */
} dmc_algo;

typedef struct dmc_ctx dmc_ctx;

typedef struct {
    const void *data;     /* host or device pointer, see the call */
    dmc_dtype dtype;
    uint32_t dims[3];     /* points along x, y, z */
} dmc_volume;

/* Host mesh returned by dmc_run; release with dmc_mesh_free. */
typedef struct {
    float *vertices;          /* 3 * n_vertices, xyz */
    uint32_t *quads;          /* 4 * n_quads */
    uint32_t *triangles;      /* 3 * n_triangles (2 per quad), or NULL */
    uint64_t n_vertices;
    uint64_t n_quads;
    uint64_t n_triangles;
} dmc_mesh;

/* Counters of the last extraction on a context. */
typedef struct {
    uint64_t n_vertices;
    uint64_t n_quads;
    uint64_t n_active_cells;
    uint64_t n_lut2_cells;
    uint64_t n_dropped_quads;   /* quads the reference would index with NO_VERTEX */
    float device_ms;            /* device time of the last call (events) */
    int algo;                   /* dmc_algo actually used */
    float count_ms;             /* brick path: count sweep, segment scan, emit sweep */
    float scan_ms;
    float emit_ms;
} dmc_stats;

/* Library version string. */
const char *dmc_version(void);
/* sha256 of the lookup tables compiled into the library. */
const char *dmc_tables_sha256(void);
/* Human-readable name of a status. */
const char *dmc_status_string(dmc_status s);
/* The CUDA error behind the last DMC_ERR_CUDA or DMC_ERR_OOM returned on the
 * calling thread ("cudaErrorName: description"), or "" if there was none;
 * also set when dmc_create finds no usable device.  The reference prints the
 * same before exit(1) (cuda_includes.h:13-19). */
const char *dmc_last_cuda_error(void);

/* Replaces dmc::setup_device_luts() (dmc.hpp:40, dmc.cu:713-779): creates a
 * context bound to CUDA device `device` holding its stream, lookup tables and
 * scratch memory.  No global state. */
dmc_status dmc_create(dmc_ctx **ctx, int device);

/* Replaces dmc::cleanup_device_luts() (dmc.hpp:48, dmc.cu:781-811). */
dmc_status dmc_destroy(dmc_ctx *ctx);

/* Select the kernel family for later calls on this context (default AUTO). */
dmc_status dmc_set_algo(dmc_ctx *ctx, dmc_algo algo);

/* Replaces dmc::run_dmc (dmc.hpp:56-57, dmc.cu:2069-2208).  `vol->data` is
 * HOST memory.  Copies the volume to the device, extracts, and returns the
 * mesh in host memory allocated by the library (triangles only when
 * want_triangles != 0).  num_smooth > 0 runs the reference's vertex smoothing
 * (dmc.cu:1914-1981, 2157-2169) that many times: each iteration moves the
 * crossing of every owned edge with a quad onto the split triangle of its
 * projected ring of dual vertices, then recomputes the dual vertices.  It
 * runs on the simple kernel family (the only one that keeps per-cell
 * offsets); with DMC_ALGO_BRICK selected it returns DMC_ERR_UNSUPPORTED. */
dmc_status dmc_run(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                   float iso, uint32_t num_smooth, int want_triangles, dmc_mesh *out);

/* dmc_run into caller-owned HOST buffers (no reference counterpart; same
 * extraction): vertices (3 floats each), quads (4 indices) and, when
 * h_triangles is not NULL, triangles (6 indices per quad) with the given
 * capacities in vertices / quads.  h_quads may be NULL when h_triangles is
 * not: the call then returns what dmc::run_dmc returns, vertices and
 * triangles, and quad_capacity bounds the triangles (two per quad).
 * Nothing is allocated per call, and with page-locked (pinned) buffers both
 * copies run at the full host-link rate: the form to use when meshes are
 * large or calls frequent.  When the mesh is larger than the capacities the
 * call returns DMC_ERR_OUTPUT_OVERFLOW with the needed counts in
 * *n_vertices / *n_quads; writes stay within the capacities, and the
 * buffers' contents are undefined. */
dmc_status dmc_run_into(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                        float iso, uint32_t num_smooth, float *h_vertices, uint64_t vertex_capacity,
                        uint32_t *h_quads, uint64_t quad_capacity, uint32_t *h_triangles,
                        uint64_t *n_vertices, uint64_t *n_quads);

/* Releases the buffers of a mesh returned by dmc_run. */
void dmc_mesh_free(dmc_mesh *mesh);

/* Device-memory form of dmc::run_dmc (no reference counterpart for the
 * zero-copy variant; same semantics).  `vol->data` is DEVICE memory.  Output
 * buffers are caller-owned device memory with the given capacities (in
 * vertices / quads).  d_triangles may be NULL.  On DMC_ERR_OUTPUT_OVERFLOW the
 * counts are still reported in *n_vertices / *n_quads so the caller can
 * retry; writes stay within the capacities, and the buffers' contents are
 * undefined.  With all three output pointers NULL the call only counts: it
 * returns DMC_OK with the totals and writes no mesh.  num_smooth > 0 smooths
 * as dmc_run does and needs d_quads along with d_vertices.  `stream` is a
 * cudaStream_t (NULL: the context's stream).  The call returns after the mesh
 * is complete. */
dmc_status dmc_extract_device(dmc_ctx *ctx, const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                              float iso, uint32_t num_smooth,
                              float *d_vertices, uint64_t vertex_capacity,
                              uint32_t *d_quads, uint64_t quad_capacity,
                              uint32_t *d_triangles,
                              uint64_t *n_vertices, uint64_t *n_quads, void *stream);

/* Writes a mesh in host memory as Wavefront OBJ, in the format of the
 * reference's dump_obj (dmc.cu:2238-2246): "v x y z" lines (six significant
 * digits), then "f ..." lines with 1-based indices; verts_per_face is 3
 * (triangles) or 4 (quads).  Indices out of range give DMC_ERR_INVALID_ARG
 * before anything is written. */
dmc_status dmc_write_obj(const char *path, const float *vertices, uint64_t n_vertices,
                         const uint32_t *faces, uint64_t n_faces, uint32_t verts_per_face);

/* Opt-in post-processing (no reference counterpart; the result no longer
 * has the reference's vertex numbering): drops every vertex no quad
 * references -- all edge crossings, which only serve to place the dual
 * vertices, and any unreferenced dual vertex -- keeping the others in order.
 * Kept vertices go to d_out_vertices (device, room for n_vertices, must not
 * overlap d_vertices); d_quads (4 per quad) and, if not NULL, d_triangles (6
 * per quad) are renumbered in place.  *n_out_vertices receives the count.
 * Out-of-range indices give DMC_ERR_DEVICE_CHECK. */
dmc_status dmc_compact_mesh(dmc_ctx *ctx, const float *d_vertices, uint64_t n_vertices,
                            uint32_t *d_quads, uint64_t n_quads, uint32_t *d_triangles,
                            float *d_out_vertices, uint64_t *n_out_vertices, void *stream);

/* Counters of the last call on this context (for a batch: summed over its
 * volumes). */
dmc_status dmc_get_stats(const dmc_ctx *ctx, dmc_stats *stats);

/* ---- batched extraction (no reference counterpart: the reference extracts
 * one volume per run_dmc call, dmc.cu:2069-2208, with a host round trip per
 * kernel) ------------------------------------------------------------------ */

/* One volume of a batch.  vol.data is DEVICE memory. */
typedef struct {
    dmc_volume vol;
    float iso;
    float xyz_min[3];
    float xyz_max[3];
} dmc_batch_item;

/* Where the mesh of one volume landed in the shared output buffers: vertices
 * [vertex_offset, vertex_offset + n_vertices), quads (and triangle pairs)
 * [quad_offset, quad_offset + n_quads).  Quad and triangle corner indices are
 * relative to the volume's vertex_offset, so each volume's slice is the mesh
 * dmc_extract_device returns for it alone. */
typedef struct {
    uint64_t vertex_offset;
    uint64_t n_vertices;
    uint64_t quad_offset;
    uint64_t n_quads;
} dmc_batch_result;

/* dmc_extract_batch flags */
#define DMC_BATCH_ASYNC 0x1u  /* enqueue and return; dmc_batch_wait completes the call */
#define DMC_BATCH_GRAPH 0x2u  /* as ASYNC, launched as a CUDA graph cached on the context */

/* Extracts n_items volumes (mixed dtypes and shapes) in one pipeline: one
 * persistent count sweep per dtype over the bricks of all volumes, one scan,
 * one persistent emit sweep per dtype.  Meshes are concatenated in item order
 * into the caller's device buffers; per-volume offsets go to d_results
 * (device, may be NULL) and, for a synchronous call, to results (host, may be
 * NULL).
 *
 * flags == 0: returns when the meshes are complete, with the totals in
 * *n_vertices / *n_quads; DMC_ERR_OUTPUT_OVERFLOW (totals and results still
 * reported; every write stays within the capacities, but the buffers' contents
 * are undefined) when they exceed the capacities.  With all
 * three output pointers NULL the call only counts: DMC_OK, totals and
 * per-volume results, no mesh.  DMC_BATCH_ASYNC / DMC_BATCH_GRAPH: enqueue on
 * `stream` and return at once; results, n_vertices and n_quads may be NULL and
 * are ignored.  Capacities are then checked on the device (writes beyond them
 * are skipped and reported by dmc_batch_wait), so size the buffers by a bound.
 * One asynchronous batch may be in flight per context: call dmc_batch_wait
 * before the next call on the context.  The graph is captured on first use and
 * again whenever the scratch layout changes; later batches of any shape that
 * fit the scratch replay it, with the output buffers of each call patched
 * into the graph.  The first call of a context allocates its scratch; a
 * batch larger than any before grows it. */
dmc_status dmc_extract_batch(dmc_ctx *ctx, const dmc_batch_item *items, uint32_t n_items,
                             float *d_vertices, uint64_t vertex_capacity,
                             uint32_t *d_quads, uint64_t quad_capacity,
                             uint32_t *d_triangles,
                             dmc_batch_result *d_results, dmc_batch_result *results,
                             uint64_t *n_vertices, uint64_t *n_quads,
                             uint32_t flags, void *stream);

/* Completes the asynchronous batch of the context: waits for it, fills
 * results (host, may be NULL) and the totals, and returns its status. */
dmc_status dmc_batch_wait(dmc_ctx *ctx, dmc_batch_result *results, uint64_t *n_vertices, uint64_t *n_quads);

/* ---- sharded extraction of one volume across ranks (no reference
 * counterpart) ------------------------------------------------------------
 *
 * The volume's cell planes are split into z ranges, one per rank (one GPU
 * each).  Rank r holds its cell planes [z_begin, z_end) of a volume with nz
 * point planes, as the point planes [max(z_begin - 1, 0), min(z_end + 3, nz))
 * in its own device memory: `local` describes them (dims[0], dims[1] those
 * of the volume, dims[2] the local plane count).  The planes beyond its cells
 * are halo: one below for the 2B/3B test of its first plane, and above, the
 * next rank's first cell plane (whose offsets the quads of its last plane
 * reference) with its 2B/3B test.
 *
 * dmc_shard_count counts the rank's part and returns its vertex and quad
 * totals.  The ranks exchange them (an exclusive scan: the vertices and quads
 * of all earlier ranks), and dmc_shard_emit writes the part into device
 * buffers: vertices and quads (triangles optional) at local positions, quad
 * indices global (local vertex index + vertex_offset).  Concatenated in rank
 * order the parts equal the unsharded mesh bit for bit.  The emit must follow
 * the count on the same context, with the local planes unchanged; on too
 * small buffers it returns DMC_ERR_OUTPUT_OVERFLOW with undefined contents. */
dmc_status dmc_shard_count(dmc_ctx *ctx, const dmc_volume *local, uint32_t nz, uint32_t z_begin, uint32_t z_end,
                           const float xyz_min[3], const float xyz_max[3], float iso,
                           uint64_t *n_vertices, uint64_t *n_quads, void *stream);
dmc_status dmc_shard_emit(dmc_ctx *ctx, uint64_t vertex_offset, float *d_vertices, uint64_t vertex_capacity,
                          uint32_t *d_quads, uint64_t quad_capacity, uint32_t *d_triangles, void *stream);

/* Tuning knobs and a test hook (no reference counterpart). */
typedef enum {
    DMC_OPT_BRICK_PLANES = 1,  /* z planes per brick, 1..256; 0 chooses from the batch size */
    DMC_OPT_STREAM_SLABS = 2,  /* dmc_run_into in z slabs (upload, extraction and download
                                  overlap): 0 automatic (volumes of 64 MiB and more, one slab
                                  per 96 MiB, 2..32), 1 never, 2..32 that many slabs */
    DMC_OPT_FAIL_ALLOCS = 3    /* test hook: the context's next n device allocations fail as
                                  when the device is out of memory (the call returns
                                  DMC_ERR_OOM; the buffer being grown is released); 0 off */
} dmc_option;

dmc_status dmc_set_option(dmc_ctx *ctx, dmc_option opt, int64_t value);

/* ---- serving loop (no reference counterpart) -----------------------------
 *
 * A server keeps a pool of device-resident volumes and extracts (volume,
 * isovalue) requests as they arrive.  Requests are admitted in FIFO order
 * while their worst-case output (7 vertices and 3 quads per cell) fits the
 * server's output arenas; admitted requests are batched onto `lanes`
 * concurrent pipelines (each a context with its own stream, launched as a
 * CUDA graph), so requests that arrive while others run join the next batch
 * as soon as a lane and arena space are free.  A result's device pointers
 * stay valid until dmc_server_release.  All calls are thread-safe. */
typedef struct dmc_server dmc_server;

typedef struct {
    int device;
    uint32_t lanes;            /* batches in flight at once (0: 2) */
    uint32_t max_batch;        /* requests per batch (0: 64) */
    uint64_t vertex_arena;     /* vertices the output arena holds, < 2^32 */
    uint64_t quad_arena;       /* quads (and triangle pairs) the output arena holds, < 2^32 */
    int want_triangles;
    int plain;                 /* 1: one lane, each request extracted alone by dmc_extract_device */
} dmc_server_config;

typedef struct {
    dmc_status status;
    uint64_t n_vertices;
    uint64_t n_quads;
    const float *vertices;     /* device memory, 3 * n_vertices */
    const uint32_t *quads;     /* device memory, 4 * n_quads; indices relative to vertices */
    const uint32_t *triangles; /* device memory, 6 * n_quads, or NULL */
    double t_submit, t_start, t_done;   /* seconds on the server's clock */
    uint32_t batch_size;       /* requests in the batch that served this one */
} dmc_server_result;

typedef struct {
    uint64_t submitted, completed, batches, max_batch_seen;
    uint64_t arena_peak_vertices, arena_peak_quads;
} dmc_server_stats;

dmc_status dmc_server_create(const dmc_server_config *cfg, dmc_server **server);
/* Fails requests never admitted, waits for batches in flight, frees everything. */
dmc_status dmc_server_destroy(dmc_server *server);
/* Adds a volume in DEVICE memory (owned by the caller, kept resident while the
 * server lives).  DMC_ERR_OUTPUT_OVERFLOW if its bound exceeds the arenas. */
dmc_status dmc_server_add_volume(dmc_server *server, const dmc_volume *vol, const float xyz_min[3],
                                 const float xyz_max[3], uint32_t *volume_id);
dmc_status dmc_server_submit(dmc_server *server, uint32_t volume_id, float iso, uint64_t *request_id);
/* Waits up to timeout_s for the request; DMC_ERR_TIMEOUT if it is not done.
 * The request's own status is in out->status. */
dmc_status dmc_server_wait(dmc_server *server, uint64_t request_id, double timeout_s, dmc_server_result *out);
/* Returns the request's output space to the arenas; the request id ends. */
dmc_status dmc_server_release(dmc_server *server, uint64_t request_id);
dmc_status dmc_server_get_stats(dmc_server *server, dmc_server_stats *stats);
/* Load generator: submits request i at arrival_s[i] seconds after the call
 * starts (a separate thread keeps the schedule), waits for and releases
 * each, and reports latency_s[i] = done - submit and status[i]. */
dmc_status dmc_server_replay(dmc_server *server, uint32_t n, const uint32_t *volume_ids, const float *isos,
                             const double *arrival_s, double *latency_s, dmc_status *status);

/* ---- no-allocation extraction (no reference counterpart) ----------------
 *
 * For callers that must not have the library allocate device memory: a
 * process whose device memory is held by a pool allocator that has reserved
 * what is free (a framework's caching allocator, an application heap), where
 * a cudaMalloc from a library fails or fragments the pool; and latency-bound
 * loops sharing the GPU with other streams, where cudaMalloc / cudaFree can
 * synchronise the device.  This call allocates nothing: it runs the simple
 * per-cell pipeline (10 bytes of scratch per cell) in one fixed array of the
 * library's own device memory, ~10.1 MiB per device, so it takes volumes of
 * at most DMC_NOALLOC_MAX_CELLS cells ((nx-1)(ny-1)(nz-1)); larger ones are
 * rejected with DMC_ERR_TOO_LARGE before any GPU work.
 *
 * No context: it runs on the calling thread's current device, on `stream`
 * (NULL: the legacy default stream), and returns when the mesh is complete.
 * The first call on a device (and the first after cudaDeviceReset) uploads
 * the lookup tables into the array and synchronises the device; make it
 * before any stream capture.  The array is one per
 * device: calls on the same device must not overlap (concurrent calls from
 * several host threads race on it).  Outputs and errors as in
 * dmc_extract_device (all output pointers NULL: count only). */
#define DMC_NOALLOC_MAX_CELLS 1048576u

dmc_status dmc_extract_device_noalloc(const dmc_volume *vol, const float xyz_min[3], const float xyz_max[3],
                                      float iso, float *d_vertices, uint64_t vertex_capacity,
                                      uint32_t *d_quads, uint64_t quad_capacity, uint32_t *d_triangles,
                                      uint64_t *n_vertices, uint64_t *n_quads, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DMC_GB300_H */
