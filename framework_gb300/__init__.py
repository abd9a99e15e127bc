"""GB300-native Dual Marching Cubes, drop-in for the reference's ``dmc`` API.

The reference (vcg-thin-meshgen/Framework, DMC_CUDA/DMC_CUDA/include/dmc.hpp)
exposes ``dmc::setup_device_luts()``, ``dmc::run_dmc(vertices, triangles,
grid, xyz_min, xyz_max, iso_value, num_smooth)`` and
``dmc::cleanup_device_luts()``.  This module mirrors those three calls on top
of the C ABI in include/dmc_gb300.h (library ``libdmc_gb300.so``, built from
framework_gb300/csrc by ``framework_gb300.build``), plus an object API with
device-memory, batched and serving entry points.

All extraction runs in the CUDA library; there is no CPU fallback.  Importing
works without a GPU, but every call that extracts fails loudly when the
library or a CUDA device is missing.
"""
import contextlib
import ctypes
import os

import numpy as np

from . import build as _build

__all__ = ["DMCError", "Extractor", "Server", "Mesh", "setup_device_luts", "run_dmc", "cleanup_device_luts",
           "write_obj", "load_library", "STATUS"]

STATUS = {
    0: "DMC_OK", 1: "DMC_ERR_INVALID_ARG", 2: "DMC_ERR_OOM", 3: "DMC_ERR_OUTPUT_OVERFLOW",
    4: "DMC_ERR_TIMEOUT", 5: "DMC_ERR_CUDA", 6: "DMC_ERR_UNSUPPORTED", 7: "DMC_ERR_DEVICE_CHECK",
    8: "DMC_ERR_TOO_LARGE",
}
NOALLOC_MAX_CELLS = 1048576
DTYPE = {"float32": 0, "uint16": 1}
ALGO = {"auto": 0, "simple": 1, "brick": 2}

# exported symbols of the C ABI (include/dmc_gb300.h)
ABI_SYMBOLS = [
    "dmc_version", "dmc_tables_sha256", "dmc_status_string", "dmc_last_cuda_error", "dmc_create", "dmc_destroy",
    "dmc_set_algo", "dmc_run", "dmc_run_into", "dmc_mesh_free", "dmc_extract_device", "dmc_get_stats",
    "dmc_extract_batch", "dmc_batch_wait", "dmc_set_option", "dmc_extract_device_noalloc",
    "dmc_server_create", "dmc_server_destroy", "dmc_server_add_volume", "dmc_server_submit", "dmc_server_wait",
    "dmc_server_release", "dmc_server_get_stats", "dmc_server_replay", "dmc_write_obj", "dmc_compact_mesh",
    "dmc_shard_count", "dmc_shard_emit",
]
BATCH_ASYNC, BATCH_GRAPH = 0x1, 0x2
OPT_BRICK_PLANES = 1
OPT_STREAM_SLABS = 2      # dmc_run_into in z slabs: 0 automatic, 1 never, 2..32 slabs
OPT_FAIL_ALLOCS = 3       # test hook: the context's next n device allocations fail (DMC_ERR_OOM)


class DMCError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = int(status)
        # for DMC_ERR_OOM / DMC_ERR_CUDA, the CUDA error behind it
        self.cuda_error = last_cuda_error() if self.status in (2, 5) else ""
        super().__init__("%s%s%s" % (STATUS.get(self.status, "status %d" % self.status),
                                     (": " + what) if what else "",
                                     (" (%s)" % self.cuda_error) if self.cuda_error else ""))


def last_cuda_error():
    """``dmc_last_cuda_error``: the CUDA error behind the last DMC_ERR_CUDA or
    DMC_ERR_OOM on this thread, or ""."""
    if _lib is None:            # nothing was called yet
        return ""
    return _lib.dmc_last_cuda_error().decode()


class _Volume(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int), ("dims", ctypes.c_uint32 * 3)]


class _BatchItem(ctypes.Structure):
    _fields_ = [("vol", _Volume), ("iso", ctypes.c_float), ("xyz_min", ctypes.c_float * 3),
                ("xyz_max", ctypes.c_float * 3)]


class _BatchResult(ctypes.Structure):
    _fields_ = [("vertex_offset", ctypes.c_uint64), ("n_vertices", ctypes.c_uint64),
                ("quad_offset", ctypes.c_uint64), ("n_quads", ctypes.c_uint64)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("lanes", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("vertex_arena", ctypes.c_uint64), ("quad_arena", ctypes.c_uint64),
                ("want_triangles", ctypes.c_int), ("plain", ctypes.c_int)]


class _ServerResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("n_vertices", ctypes.c_uint64), ("n_quads", ctypes.c_uint64),
                ("vertices", ctypes.c_void_p), ("quads", ctypes.c_void_p), ("triangles", ctypes.c_void_p),
                ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double), ("t_done", ctypes.c_double),
                ("batch_size", ctypes.c_uint32)]


class _ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("max_batch_seen", ctypes.c_uint64), ("arena_peak_vertices", ctypes.c_uint64),
                ("arena_peak_quads", ctypes.c_uint64)]


class _Mesh(ctypes.Structure):
    _fields_ = [("vertices", ctypes.POINTER(ctypes.c_float)), ("quads", ctypes.POINTER(ctypes.c_uint32)),
                ("triangles", ctypes.POINTER(ctypes.c_uint32)), ("n_vertices", ctypes.c_uint64),
                ("n_quads", ctypes.c_uint64), ("n_triangles", ctypes.c_uint64)]


class Stats(ctypes.Structure):
    _fields_ = [("n_vertices", ctypes.c_uint64), ("n_quads", ctypes.c_uint64),
                ("n_active_cells", ctypes.c_uint64), ("n_lut2_cells", ctypes.c_uint64),
                ("n_dropped_quads", ctypes.c_uint64), ("device_ms", ctypes.c_float), ("algo", ctypes.c_int),
                ("count_ms", ctypes.c_float), ("scan_ms", ctypes.c_float), ("emit_ms", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def library_path():
    return _build.LIB


def load_library(build_if_missing=True):
    """Load libdmc_gb300.so (building it first if needed) and declare the ABI."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or not _build.up_to_date():
        if not build_if_missing:
            raise DMCError(5, "CUDA library %s is missing; run framework_gb300.build" % path)
        _build.build()
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    L.dmc_version.restype = ctypes.c_char_p
    L.dmc_tables_sha256.restype = ctypes.c_char_p
    L.dmc_status_string.restype = ctypes.c_char_p
    L.dmc_status_string.argtypes = [ctypes.c_int]
    L.dmc_last_cuda_error.restype = ctypes.c_char_p
    L.dmc_last_cuda_error.argtypes = []
    L.dmc_create.argtypes = [P(ctypes.c_void_p), ctypes.c_int]
    L.dmc_destroy.argtypes = [ctypes.c_void_p]
    L.dmc_set_algo.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.dmc_run.argtypes = [ctypes.c_void_p, P(_Volume), P(ctypes.c_float), P(ctypes.c_float), ctypes.c_float,
                          ctypes.c_uint32, ctypes.c_int, P(_Mesh)]
    L.dmc_run_into.argtypes = [ctypes.c_void_p, P(_Volume), P(ctypes.c_float), P(ctypes.c_float), ctypes.c_float,
                               ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                               ctypes.c_void_p, P(ctypes.c_uint64), P(ctypes.c_uint64)]
    L.dmc_mesh_free.argtypes = [P(_Mesh)]
    L.dmc_mesh_free.restype = None
    L.dmc_extract_device.argtypes = [ctypes.c_void_p, P(_Volume), P(ctypes.c_float), P(ctypes.c_float), ctypes.c_float,
                                     ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                     ctypes.c_uint64, ctypes.c_void_p, P(ctypes.c_uint64), P(ctypes.c_uint64),
                                     ctypes.c_void_p]
    L.dmc_get_stats.argtypes = [ctypes.c_void_p, P(Stats)]
    L.dmc_extract_batch.argtypes = [ctypes.c_void_p, P(_BatchItem), ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint64,
                                    ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
                                    P(_BatchResult), P(ctypes.c_uint64), P(ctypes.c_uint64), ctypes.c_uint32,
                                    ctypes.c_void_p]
    L.dmc_batch_wait.argtypes = [ctypes.c_void_p, P(_BatchResult), P(ctypes.c_uint64), P(ctypes.c_uint64)]
    L.dmc_set_option.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64]
    L.dmc_shard_count.argtypes = [ctypes.c_void_p, P(_Volume), ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                  P(ctypes.c_float), P(ctypes.c_float), ctypes.c_float, P(ctypes.c_uint64),
                                  P(ctypes.c_uint64), ctypes.c_void_p]
    L.dmc_shard_emit.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                 ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    L.dmc_compact_mesh.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                   ctypes.c_void_p, ctypes.c_void_p, P(ctypes.c_uint64), ctypes.c_void_p]
    L.dmc_write_obj.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                ctypes.c_uint32]
    L.dmc_server_create.argtypes = [P(_ServerConfig), P(ctypes.c_void_p)]
    L.dmc_server_destroy.argtypes = [ctypes.c_void_p]
    L.dmc_server_add_volume.argtypes = [ctypes.c_void_p, P(_Volume), P(ctypes.c_float), P(ctypes.c_float),
                                        P(ctypes.c_uint32)]
    L.dmc_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, P(ctypes.c_uint64)]
    L.dmc_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, P(_ServerResult)]
    L.dmc_server_release.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
    L.dmc_server_get_stats.argtypes = [ctypes.c_void_p, P(_ServerStats)]
    L.dmc_server_replay.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    L.dmc_extract_device_noalloc.argtypes = [P(_Volume), P(ctypes.c_float), P(ctypes.c_float), ctypes.c_float,
                                             ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                             ctypes.c_void_p, P(ctypes.c_uint64), P(ctypes.c_uint64),
                                             ctypes.c_void_p]
    for name in ABI_SYMBOLS:
        if name not in ("dmc_version", "dmc_tables_sha256", "dmc_status_string", "dmc_last_cuda_error", "dmc_mesh_free"):
            getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


def _f3(v):
    return (ctypes.c_float * 3)(*[float(x) for x in v])


def _check(status, what=""):
    if status != 0:
        raise DMCError(status, what)


class _MeshBuffers:
    """Owns the host buffers of one dmc_run mesh.  Each numpy array handed out
    keeps this object alive through its buffer, so dmc_mesh_free runs when
    the last of them is collected."""

    def __init__(self, lib, mesh):
        self._lib, self._mesh = lib, mesh

    def array(self, ptr, ctype, rows, cols):
        n = rows * cols
        if n == 0:
            return np.zeros((0, cols), dtype=np.dtype(ctype))
        buf = (ctype * n).from_address(ctypes.addressof(ptr.contents))
        buf._owner = self
        return np.frombuffer(buf, dtype=np.dtype(ctype)).reshape(rows, cols)

    def __del__(self):
        try:
            self._lib.dmc_mesh_free(ctypes.byref(self._mesh))
        except Exception:
            pass


class Mesh:
    """Extraction result in host memory: vertices (V,3) float32, quads (Q,4)
    uint32 and, when requested, triangles (2Q,3) uint32 in the reference's
    split (q0,q1,q2), (q2,q3,q0)."""

    def __init__(self, vertices, quads, triangles=None, stats=None):
        self.vertices = vertices
        self.quads = quads
        self.triangles = triangles
        self.stats = stats or {}

    def __repr__(self):
        return "Mesh(V=%d, Q=%d)" % (len(self.vertices), len(self.quads))


def _volume_struct(data_ptr, dtype, dims):
    v = _Volume()
    v.data = data_ptr
    v.dtype = dtype
    v.dims[0], v.dims[1], v.dims[2] = [int(d) for d in dims]
    return v


def _host_volume(volume):
    arr = np.ascontiguousarray(volume)
    if arr.ndim != 3:
        raise DMCError(1, "volume must be a 3-D array indexed [z, y, x]")
    if arr.dtype == np.float32:
        dt = 0
    elif arr.dtype == np.uint16:
        dt = 1
    else:
        raise DMCError(1, "volume dtype must be float32 or uint16, got %s" % arr.dtype)
    nz, ny, nx = arr.shape
    return arr, _volume_struct(arr.ctypes.data, dt, (nx, ny, nz))


def _default_extent(dims_xyz, xyz_min, xyz_max):
    if xyz_min is None:
        xyz_min = (0.0, 0.0, 0.0)
    if xyz_max is None:
        xyz_max = tuple(float(d - 1) for d in dims_xyz)
    return xyz_min, xyz_max


class Extractor:
    """One extraction context on one CUDA device (``dmc_create``)."""

    def __init__(self, device=0, algo="auto"):
        self._lib = load_library()
        h = ctypes.c_void_p()
        _check(self._lib.dmc_create(ctypes.byref(h), int(device)), "dmc_create(device=%d)" % device)
        self._h = h
        self.device = int(device)
        self.set_algo(algo)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.dmc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_algo(self, algo):
        _check(self._lib.dmc_set_algo(self._h, ALGO[algo] if isinstance(algo, str) else int(algo)))

    def stats(self):
        s = Stats()
        _check(self._lib.dmc_get_stats(self._h, ctypes.byref(s)))
        return s.as_dict()

    def run(self, volume, xyz_min=None, xyz_max=None, iso=0.0, num_smooth=0, triangles=True):
        """Host-memory extraction (``dmc_run``): numpy [z,y,x] float32/uint16 in, Mesh out."""
        arr, vol = _host_volume(volume)
        mn, mx = _default_extent(vol.dims, xyz_min, xyz_max)
        m = _Mesh()
        _check(self._lib.dmc_run(self._h, ctypes.byref(vol), _f3(mn), _f3(mx), ctypes.c_float(iso),
                                 int(num_smooth), 1 if triangles else 0, ctypes.byref(m)), "dmc_run")
        # the arrays wrap the library's buffers (no copy); they are released
        # with dmc_mesh_free once the last array referring to them is gone
        owner = _MeshBuffers(self._lib, m)
        V, Q = int(m.n_vertices), int(m.n_quads)
        verts = owner.array(m.vertices, ctypes.c_float, V, 3)
        quads = owner.array(m.quads, ctypes.c_uint32, Q, 4)
        tris = owner.array(m.triangles, ctypes.c_uint32, 2 * Q, 3) if triangles else None
        return Mesh(verts, quads, tris, self.stats())

    def run_into(self, volume, vertices, quads, triangles=None, xyz_min=None, xyz_max=None, iso=0.0, num_smooth=0):
        """Host-memory extraction into caller buffers (``dmc_run_into``).

        ``volume`` is a numpy [z,y,x] float32/uint16 array; ``vertices``
        (float32 [V,3]), ``quads`` (uint32/int32 [Q,4]) and ``triangles``
        ([2Q,3] or None) are host arrays, e.g. numpy views of pinned torch
        tensors.  ``quads`` may be None when ``triangles`` is given: the
        reference's outputs, vertices and triangles.  Returns (n_vertices,
        n_quads); raises DMCError carrying the needed counts in ``.counts``
        when the buffers are too small."""
        arr, vol = _host_volume(volume)
        mn, mx = _default_extent(vol.dims, xyz_min, xyz_max)
        if quads is None and triangles is None:
            raise DMCError(1, "run_into needs a quad or a triangle buffer")
        for name, b in (("vertices", vertices), ("quads", quads), ("triangles", triangles)):
            if b is not None and not b.flags["C_CONTIGUOUS"]:
                raise DMCError(1, "%s must be C-contiguous" % name)
        caps = ([quads.size // 4] if quads is not None else []) + ([triangles.size // 6] if triangles is not None else [])
        qcap = min(caps)
        nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
        rc = self._lib.dmc_run_into(self._h, ctypes.byref(vol), _f3(mn), _f3(mx), ctypes.c_float(iso), int(num_smooth),
                                    vertices.ctypes.data, vertices.size // 3,
                                    quads.ctypes.data if quads is not None else None, qcap,
                                    triangles.ctypes.data if triangles is not None else None,
                                    ctypes.byref(nv), ctypes.byref(nq))
        if rc != 0:
            e = DMCError(rc, "dmc_run_into")
            e.counts = (int(nv.value), int(nq.value))
            raise e
        return int(nv.value), int(nq.value)

    def extract_device(self, volume, xyz_min=None, xyz_max=None, iso=0.0, vertices=None, quads=None,
                       triangles=None, stream=None, dims=None, dtype=None, num_smooth=0):
        """Device-memory extraction (``dmc_extract_device``).

        ``volume`` is a CUDA tensor [z,y,x] (float32, or int16 holding uint16
        bit patterns) or a raw device pointer with ``dims``/``dtype``.  Output
        buffers are CUDA tensors (float32 [V,3], int32/uint32 [Q,4]); returns
        (n_vertices, n_quads).  Raises DMCError(OUTPUT_OVERFLOW) carrying the
        needed counts in ``.counts`` when the buffers are too small; with no
        output buffers at all it only counts."""
        if isinstance(volume, int):
            ptr, dims_xyz, dt = volume, dims, DTYPE[dtype]
        else:
            t = volume
            if not t.is_cuda or not t.is_contiguous() or t.dim() != 3:
                raise DMCError(1, "volume must be a contiguous 3-D CUDA tensor")
            name = str(t.dtype).replace("torch.", "")
            dt = {"float32": 0, "int16": 1, "uint16": 1}.get(name)
            if dt is None:
                raise DMCError(1, "volume tensor dtype must be float32 or (u)int16")
            ptr = t.data_ptr()
            dims_xyz = (t.shape[2], t.shape[1], t.shape[0])
        vol = _volume_struct(ptr, dt, dims_xyz)
        mn, mx = _default_extent(vol.dims, xyz_min, xyz_max)
        vptr = vertices.data_ptr() if vertices is not None else None
        vcap = vertices.numel() // 3 if vertices is not None else 0
        qptr = quads.data_ptr() if quads is not None else None
        qcap = quads.numel() // 4 if quads is not None else 0
        tptr = triangles.data_ptr() if triangles is not None else None
        if triangles is not None:
            qcap = min(qcap, triangles.numel() // 6)
        nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
        st = _stream_handle(stream)
        rc = self._lib.dmc_extract_device(self._h, ctypes.byref(vol), _f3(mn), _f3(mx), ctypes.c_float(iso),
                                          int(num_smooth),
                                          vptr, vcap, qptr, qcap, tptr, ctypes.byref(nv), ctypes.byref(nq), st)
        if rc != 0:
            e = DMCError(rc, "dmc_extract_device")
            e.counts = (int(nv.value), int(nq.value))
            raise e
        return int(nv.value), int(nq.value)

    def compact_mesh(self, vertices, quads, triangles=None, out_vertices=None, stream=None):
        """``dmc_compact_mesh``: keep only the vertices the quads reference.

        ``vertices`` (CUDA float32 [V,3]) is read; ``quads`` (CUDA int32 [Q,4])
        and ``triangles`` ([2Q,3]) are renumbered in place.  Returns the kept
        vertices as a view of ``out_vertices`` (allocated when not given)."""
        import torch
        if out_vertices is None:
            out_vertices = torch.empty_like(vertices)
        n = ctypes.c_uint64()
        _check(self._lib.dmc_compact_mesh(self._h, vertices.data_ptr(), vertices.shape[0], quads.data_ptr(),
                                          quads.shape[0], triangles.data_ptr() if triangles is not None else None,
                                          out_vertices.data_ptr(), ctypes.byref(n), _stream_handle(stream)),
               "dmc_compact_mesh")
        return out_vertices[:int(n.value)]

    def shard_count(self, local, nz, z_begin, z_end, xyz_min=None, xyz_max=None, iso=0.0, stream=None):
        """``dmc_shard_count``: this rank's part of a sharded extraction.

        ``local`` is a contiguous CUDA tensor [planes, y, x] (float32, or int16
        holding uint16 bit patterns) with the point planes
        ``shard.point_planes(nz, z_begin, z_end)`` of a volume with ``nz``
        point planes; ``z_begin`` / ``z_end`` are cell planes of the whole
        volume, whose default extent is (0, 0, 0)..(x-1, y-1, nz-1).  Returns
        this rank's (n_vertices, n_quads)."""
        t = local
        if not t.is_cuda or not t.is_contiguous() or t.dim() != 3:
            raise DMCError(1, "local planes must be a contiguous 3-D CUDA tensor")
        dt = {"float32": 0, "int16": 1, "uint16": 1}.get(str(t.dtype).replace("torch.", ""))
        if dt is None:
            raise DMCError(1, "volume tensor dtype must be float32 or (u)int16")
        vol = _volume_struct(t.data_ptr(), dt, (t.shape[2], t.shape[1], t.shape[0]))
        mn, mx = _default_extent((t.shape[2], t.shape[1], nz), xyz_min, xyz_max)
        nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.dmc_shard_count(self._h, ctypes.byref(vol), int(nz), int(z_begin), int(z_end), _f3(mn),
                                         _f3(mx), ctypes.c_float(iso), ctypes.byref(nv), ctypes.byref(nq),
                                         _stream_handle(stream)), "dmc_shard_count")
        return int(nv.value), int(nq.value)

    def shard_emit(self, vertex_offset, vertices, quads, triangles=None, stream=None):
        """``dmc_shard_emit``: writes the part counted by ``shard_count`` into
        CUDA tensors (float32 [V,3], int32/uint32 [Q,4], optional [2Q,3]),
        quad indices offset by ``vertex_offset`` (the vertices of all earlier
        ranks)."""
        qcap = quads.numel() // 4
        if triangles is not None:
            qcap = min(qcap, triangles.numel() // 6)
        _check(self._lib.dmc_shard_emit(self._h, int(vertex_offset), vertices.data_ptr(), vertices.numel() // 3,
                                        quads.data_ptr(), qcap,
                                        triangles.data_ptr() if triangles is not None else None,
                                        _stream_handle(stream)), "dmc_shard_emit")

    def set_option(self, option, value):
        """``dmc_set_option``: e.g. ``set_option(OPT_BRICK_PLANES, 16)``; 0 restores the automatic choice."""
        _check(self._lib.dmc_set_option(self._h, int(option), int(value)), "dmc_set_option")

    def extract_batch(self, volumes, vertices=None, quads=None, triangles=None, results=None, mode="sync",
                      stream=None):
        """Batched device-memory extraction (``dmc_extract_batch``).

        ``volumes`` is a list of dicts with ``volume`` (CUDA tensor [z,y,x],
        float32 or (u)int16 holding uint16 bits), ``iso`` and optional
        ``xyz_min`` / ``xyz_max``.  ``results`` is an optional CUDA int64
        tensor [n, 4] that receives (vertex_offset, n_vertices, quad_offset,
        n_quads) per volume on the device.  ``mode`` "sync" returns
        (n_vertices, n_quads, host results as an (n, 4) uint64 array);
        "async" and "graph" enqueue on ``stream`` and return None:
        ``batch_wait()`` then returns the same triple."""
        n = len(volumes)
        items = (_BatchItem * n)()
        self._batch_keep = []
        for i, d in enumerate(volumes):
            t = d["volume"]
            if not t.is_cuda or not t.is_contiguous() or t.dim() != 3:
                raise DMCError(1, "batch volume %d must be a contiguous 3-D CUDA tensor" % i)
            dt = {"float32": 0, "int16": 1, "uint16": 1}.get(str(t.dtype).replace("torch.", ""))
            if dt is None:
                raise DMCError(1, "batch volume %d dtype must be float32 or (u)int16" % i)
            dims = (t.shape[2], t.shape[1], t.shape[0])
            mn, mx = _default_extent(dims, d.get("xyz_min"), d.get("xyz_max"))
            items[i].vol = _volume_struct(t.data_ptr(), dt, dims)
            items[i].iso = float(d.get("iso", 0.0))
            for k in range(3):
                items[i].xyz_min[k] = float(mn[k])
                items[i].xyz_max[k] = float(mx[k])
        vptr = vertices.data_ptr() if vertices is not None else None
        vcap = vertices.numel() // 3 if vertices is not None else 0
        qptr = quads.data_ptr() if quads is not None else None
        qcap = quads.numel() // 4 if quads is not None else 0
        tptr = triangles.data_ptr() if triangles is not None else None
        if triangles is not None:
            qcap = min(qcap, triangles.numel() // 6)
        rptr = None
        if results is not None:
            if not results.is_cuda or results.numel() < 4 * n or results.element_size() != 8:
                raise DMCError(1, "results must be a CUDA 64-bit tensor with 4 entries per volume")
            rptr = results.data_ptr()
        st = _stream_handle(stream)
        flags = {"sync": 0, "async": BATCH_ASYNC, "graph": BATCH_GRAPH}[mode]
        hres = (_BatchResult * n)()
        nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
        rc = self._lib.dmc_extract_batch(self._h, items, n, vptr, vcap, qptr, qcap, tptr, rptr, hres,
                                         ctypes.byref(nv), ctypes.byref(nq), flags, st)
        self._batch_n = n
        if rc != 0:
            e = DMCError(rc, "dmc_extract_batch")
            e.counts = (int(nv.value), int(nq.value))
            raise e
        if flags:
            return None
        return int(nv.value), int(nq.value), _results_array(hres)

    def batch_wait(self):
        """``dmc_batch_wait``: completes an async/graph batch; returns (n_vertices, n_quads, results)."""
        n = getattr(self, "_batch_n", 0)
        hres = (_BatchResult * max(n, 1))()
        nv, nq = ctypes.c_uint64(), ctypes.c_uint64()
        rc = self._lib.dmc_batch_wait(self._h, hres, ctypes.byref(nv), ctypes.byref(nq))
        if rc != 0:
            e = DMCError(rc, "dmc_batch_wait")
            e.counts = (int(nv.value), int(nq.value))
            raise e
        return int(nv.value), int(nq.value), _results_array(hres)[:n]


_CUDA_STREAM_LEGACY = 0x1   # cudaStreamLegacy: the legacy default stream


def _stream_handle(stream):
    """cudaStream_t for the C ABI.  None: torch's current stream, so the work
    is ordered after whatever torch queued there.  The C ABI reads a NULL
    handle as the context's own stream, so torch's legacy default stream
    (handle 0) is passed as cudaStreamLegacy."""
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    st = stream.cuda_stream if hasattr(stream, "cuda_stream") else stream
    st = int(st or 0)
    return st if st else _CUDA_STREAM_LEGACY


def _results_array(hres):
    return np.array([[r.vertex_offset, r.n_vertices, r.quad_offset, r.n_quads] for r in hres], dtype=np.uint64).reshape(-1, 4)


class Server:
    """Serving loop (``dmc_server_*``): a pool of device-resident volumes and
    continuous batching of (volume, isovalue) requests.

    ``vertex_arena`` / ``quad_arena`` size the output space shared by all
    requests in flight or not yet released; a request is admitted when its
    worst-case output (7 vertices, 3 quads per cell) fits.  ``plain=True``
    serves each request alone with ``dmc_extract_device`` (the per-request
    baseline)."""

    def __init__(self, device=0, vertex_arena=1 << 28, quad_arena=1 << 27, lanes=2, max_batch=64,
                 triangles=False, plain=False):
        self._lib = load_library()
        cfg = _ServerConfig(int(device), int(lanes), int(max_batch), int(vertex_arena), int(quad_arena),
                            1 if triangles else 0, 1 if plain else 0)
        h = ctypes.c_void_p()
        _check(self._lib.dmc_server_create(ctypes.byref(cfg), ctypes.byref(h)), "dmc_server_create")
        self._h = h
        self._volumes = []          # keep the pool's tensors alive

    def close(self):
        if getattr(self, "_h", None):
            self._lib.dmc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def add_volume(self, volume, xyz_min=None, xyz_max=None):
        """Adds a CUDA tensor [z,y,x] (float32, or int16 holding uint16 bits) to the pool; returns its id."""
        t = volume
        if not t.is_cuda or not t.is_contiguous() or t.dim() != 3:
            raise DMCError(1, "pool volume must be a contiguous 3-D CUDA tensor")
        dt = {"float32": 0, "int16": 1, "uint16": 1}.get(str(t.dtype).replace("torch.", ""))
        if dt is None:
            raise DMCError(1, "pool volume dtype must be float32 or (u)int16")
        dims = (t.shape[2], t.shape[1], t.shape[0])
        mn, mx = _default_extent(dims, xyz_min, xyz_max)
        vol = _volume_struct(t.data_ptr(), dt, dims)
        vid = ctypes.c_uint32()
        _check(self._lib.dmc_server_add_volume(self._h, ctypes.byref(vol), _f3(mn), _f3(mx), ctypes.byref(vid)),
               "dmc_server_add_volume")
        self._volumes.append(t)
        return int(vid.value)

    def submit(self, volume_id, iso):
        rid = ctypes.c_uint64()
        _check(self._lib.dmc_server_submit(self._h, int(volume_id), ctypes.c_float(iso), ctypes.byref(rid)),
               "dmc_server_submit")
        return int(rid.value)

    def wait(self, request_id, timeout=60.0):
        """Returns a dict with status, counts, device pointers and timestamps."""
        r = _ServerResult()
        _check(self._lib.dmc_server_wait(self._h, int(request_id), float(timeout), ctypes.byref(r)),
               "dmc_server_wait")
        return dict(status=int(r.status), n_vertices=int(r.n_vertices), n_quads=int(r.n_quads),
                    vertices=r.vertices, quads=r.quads, triangles=r.triangles, t_submit=r.t_submit,
                    t_start=r.t_start, t_done=r.t_done, batch_size=int(r.batch_size))

    def tensors(self, result):
        """Zero-copy CUDA tensors over a result's mesh (vertices [V,3] f32,
        quads [Q,4] int32, triangles [2Q,3] int32 or None); valid until the
        request is released."""
        import torch
        nv, nq = result["n_vertices"], result["n_quads"]

        def view(ptr, shape, typestr):
            if not shape[0]:
                return torch.empty(shape, dtype=torch.float32 if typestr == "<f4" else torch.int32, device="cuda")
            return torch.as_tensor(_DeviceArray(ptr, shape, typestr), device="cuda")
        v = view(result["vertices"], (nv, 3), "<f4")
        q = view(result["quads"], (nq, 4), "<i4")
        t = view(result["triangles"], (2 * nq, 3), "<i4") if result["triangles"] else None
        return v, q, t

    def fetch(self, result):
        """Host copies of a result's mesh: (vertices, quads, triangles or None) as numpy arrays."""
        v, q, t = self.tensors(result)
        return v.cpu().numpy(), q.cpu().numpy().view(np.uint32), (t.cpu().numpy().view(np.uint32) if t is not None else None)

    def fetch_into(self, result, vertices, quads, triangles=None, stream=None):
        """Copies a result's mesh into caller-owned host buffers: numpy
        arrays or CPU tensors with at least (V, 3) / (Q, 4) / (2Q, 3) rows.
        Page-locked ones (e.g. numpy views of pinned torch tensors) copy at
        the full host-link rate, and nothing is allocated per call.  Returns
        (n_vertices, n_quads); raises DMCError(OUTPUT_OVERFLOW) with
        ``.counts`` when a buffer is too small.

        With ``stream`` (a torch.cuda.Stream) the copies are only enqueued
        there, after the work already queued on it: the call returns at once,
        and the caller synchronises the stream (or an event recorded on it)
        before it reads the buffers or releases the request, whose device
        memory the copies read."""
        import torch
        v, q, t = self.tensors(result)
        nv, nq = v.shape[0], q.shape[0]
        if len(vertices) < nv or len(quads) < nq or (triangles is not None and t is not None and len(triangles) < 2 * nq):
            e = DMCError(3, "fetch_into")
            e.counts = (nv, nq)
            raise e

        def host(a, dtype):
            # same bits, as the device tensor's dtype (uint32 arrays as int32)
            if isinstance(a, torch.Tensor):
                return a.view(dtype)
            return torch.from_numpy(a.view(np.float32 if dtype == torch.float32 else np.int32))
        nb = stream is not None
        with torch.cuda.stream(stream) if nb else contextlib.nullcontext():
            if nv:
                host(vertices, torch.float32)[:nv].copy_(v, non_blocking=nb)
            if nq:
                host(quads, torch.int32)[:nq].copy_(q, non_blocking=nb)
                if triangles is not None and t is not None:
                    host(triangles, torch.int32)[:2 * nq].copy_(t, non_blocking=nb)
        return nv, nq

    def release(self, request_id):
        _check(self._lib.dmc_server_release(self._h, int(request_id)), "dmc_server_release")

    def stats(self):
        s = _ServerStats()
        _check(self._lib.dmc_server_get_stats(self._h, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in _ServerStats._fields_}

    def replay(self, volume_ids, isos, arrivals):
        """Load generator (``dmc_server_replay``): returns (latency seconds, statuses) as numpy arrays."""
        n = len(volume_ids)
        vids = np.ascontiguousarray(volume_ids, np.uint32)
        iso = np.ascontiguousarray(isos, np.float32)
        arr = np.ascontiguousarray(arrivals, np.float64)
        lat = np.zeros(n, np.float64)
        st = np.zeros(n, np.int32)
        _check(self._lib.dmc_server_replay(self._h, n, vids.ctypes.data, iso.ctypes.data, arr.ctypes.data,
                                           lat.ctypes.data, st.ctypes.data), "dmc_server_replay")
        return lat, st


class _DeviceArray:
    """__cuda_array_interface__ over library-owned device memory."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 2, "strides": None}


def write_obj(path, vertices, faces):
    """``dmc_write_obj``: vertices (V,3) float32 and triangles (T,3) or quads
    (Q,4) uint32 in host memory to a Wavefront OBJ file, in the reference's
    dump_obj format (dmc.cu:2238-2246)."""
    L = load_library()
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    f = np.ascontiguousarray(faces, np.uint32)
    if f.ndim != 2 or f.shape[1] not in (3, 4):
        raise DMCError(1, "faces must be (n, 3) or (n, 4)")
    _check(L.dmc_write_obj(os.fsencode(path), v.ctypes.data, v.shape[0], f.ctypes.data, f.shape[0], f.shape[1]),
           "dmc_write_obj")


# ---------------------------------------------------------------------------
# reference-shaped module API (dmc.hpp:40-57)

_default = None


def setup_device_luts(device=0):
    """``dmc::setup_device_luts()``: create the process-wide default context."""
    global _default
    if _default is None:
        _default = Extractor(device)
    return _default


def cleanup_device_luts():
    """``dmc::cleanup_device_luts()``: release the default context."""
    global _default
    if _default is not None:
        _default.close()
        _default = None


def run_dmc(scalar_grid, xyz_min, xyz_max, iso_value, num_smooth=0):
    """``dmc::run_dmc``: returns (vertices float32 (V,3), triangles uint32 (T,3)).

    ``scalar_grid`` is indexed [z, y, x] (utils::Array3D layout)."""
    ctx = setup_device_luts()
    m = ctx.run(scalar_grid, xyz_min, xyz_max, iso_value, num_smooth=num_smooth, triangles=True)
    return m.vertices, m.triangles
