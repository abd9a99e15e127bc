"""Ownership of dmc_run's mesh in Python (no GPU needed): Extractor.run wraps
the library's malloc'd buffers in numpy arrays without copying, and
dmc_mesh_free runs exactly once, after the last array that refers to any of
the buffers is gone.  A fake library records the free."""
import ctypes
import gc

import numpy as np

import framework_gb300 as fg


class _FakeLib:
    def __init__(self):
        self.freed = 0

    def dmc_mesh_free(self, mesh_ref):
        self.freed += 1


def _mesh(V, Q):
    verts = (ctypes.c_float * (3 * V))(*[float(i) for i in range(3 * V)])
    quads = (ctypes.c_uint32 * (4 * Q))(*range(4 * Q))
    tris = (ctypes.c_uint32 * (6 * Q))(*range(6 * Q))
    m = fg._Mesh()
    m.vertices = ctypes.cast(verts, ctypes.POINTER(ctypes.c_float))
    m.quads = ctypes.cast(quads, ctypes.POINTER(ctypes.c_uint32))
    m.triangles = ctypes.cast(tris, ctypes.POINTER(ctypes.c_uint32))
    m.n_vertices, m.n_quads, m.n_triangles = V, Q, 2 * Q
    return m, (verts, quads, tris)


def test_arrays_share_the_buffers_and_free_once():
    lib = _FakeLib()
    m, keep = _mesh(5, 3)
    owner = fg._MeshBuffers(lib, m)
    v = owner.array(m.vertices, ctypes.c_float, 5, 3)
    q = owner.array(m.quads, ctypes.c_uint32, 3, 4)
    t = owner.array(m.triangles, ctypes.c_uint32, 6, 3)
    del owner
    gc.collect()
    assert lib.freed == 0
    assert v.dtype == np.float32 and v.shape == (5, 3) and q.dtype == np.uint32 and t.shape == (6, 3)
    assert np.array_equal(v.ravel(), np.arange(15, dtype=np.float32)) and np.array_equal(q.ravel(), np.arange(12))
    assert not v.flags["OWNDATA"] and v.ctypes.data == ctypes.addressof(keep[0])   # no copy
    sub = q[1:]
    del v, q, t
    gc.collect()
    assert lib.freed == 0                      # a view of one array still holds the buffers
    del sub
    gc.collect()
    assert lib.freed == 1


def test_empty_mesh_arrays():
    lib = _FakeLib()
    m, keep = _mesh(0, 0)
    owner = fg._MeshBuffers(lib, m)
    v = owner.array(m.vertices, ctypes.c_float, 0, 3)
    q = owner.array(m.quads, ctypes.c_uint32, 0, 4)
    assert v.shape == (0, 3) and v.dtype == np.float32 and q.shape == (0, 4) and q.dtype == np.uint32
    del owner, v, q
    gc.collect()
    assert lib.freed == 1
