"""CPU oracle for Dual Marching Cubes (test infrastructure only).

A ctypes front end over ``dmc_oracle.c``, the sequential C restatement of the
reference's ``dmc::run_dmc`` (DMC_CUDA/DMC_CUDA/src/dmc.cu:2069-2208).  Only
tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline import this
package; the product never does.
"""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("vertices", ctypes.POINTER(ctypes.c_float)),
        ("vertices64", ctypes.POINTER(ctypes.c_double)),
        ("quads", ctypes.POINTER(ctypes.c_uint32)),
        ("n_vertices", ctypes.c_uint64),
        ("n_quads", ctypes.c_uint64),
        ("n_active", ctypes.c_uint64),
        ("n_lut2", ctypes.c_uint64),
        ("n_dropped_quads", ctypes.c_uint64),
        ("n_iso_samples", ctypes.c_uint64),
        ("ownerless", ctypes.POINTER(ctypes.c_uint8)),
    ]


def lib():
    global _lib
    if _lib is None:
        so = build_oracle.build()
        L = ctypes.CDLL(so)
        L.oracle_dmc.restype = ctypes.c_int
        L.oracle_dmc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32),
                                 ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                 ctypes.c_float, ctypes.c_int, ctypes.POINTER(_Mesh)]
        L.oracle_dmc_ex.restype = ctypes.c_int
        L.oracle_dmc_ex.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32),
                                    ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                    ctypes.c_float, ctypes.c_int, ctypes.c_uint32, ctypes.POINTER(_Mesh)]
        L.oracle_free.argtypes = [ctypes.POINTER(_Mesh)]
        L.oracle_free.restype = None
        L.oracle_tables_sha256.restype = ctypes.c_char_p
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_set_threads.restype = None
        _lib = L
    return _lib


def tables_sha256():
    return lib().oracle_tables_sha256().decode()


def set_threads(n):
    lib().oracle_set_threads(int(n))


def extract(volume, xyz_min=None, xyz_max=None, iso=0.0, precision=0, num_smooth=0):
    """Run the oracle on ``volume`` (numpy array indexed [z, y, x], float32 or uint16).

    ``xyz_min``/``xyz_max`` default to 0 and dims-1 (unit spacing).  Returns a dict
    with ``vertices`` (V x 3, float32 or float64), ``quads`` (Q x 4, uint32),
    ``triangles`` (2Q x 3: (q0,q1,q2), (q2,q3,q0) per quad) and counters.
    """
    vol = np.ascontiguousarray(volume)
    if vol.dtype == np.float32:
        dtype = 0
    elif vol.dtype == np.uint16:
        dtype = 1
    else:
        raise TypeError("volume must be float32 or uint16")
    nz, ny, nx = vol.shape
    dims = (ctypes.c_uint32 * 3)(nx, ny, nz)
    if xyz_min is None:
        xyz_min = (0.0, 0.0, 0.0)
    if xyz_max is None:
        xyz_max = (float(nx - 1), float(ny - 1), float(nz - 1))
    mn = (ctypes.c_float * 3)(*[float(v) for v in xyz_min])
    mx = (ctypes.c_float * 3)(*[float(v) for v in xyz_max])
    m = _Mesh()
    rc = lib().oracle_dmc_ex(vol.ctypes.data, dtype, dims, mn, mx, ctypes.c_float(iso), int(precision),
                             int(num_smooth), ctypes.byref(m))
    if rc != 0:
        raise RuntimeError("oracle_dmc failed with code %d" % rc)
    try:
        V, Q = int(m.n_vertices), int(m.n_quads)
        if precision == 0:
            verts = np.ctypeslib.as_array(m.vertices, shape=(V * 3,)).copy().reshape(V, 3) if V else np.zeros((0, 3), np.float32)
        else:
            verts = np.ctypeslib.as_array(m.vertices64, shape=(V * 3,)).copy().reshape(V, 3) if V else np.zeros((0, 3), np.float64)
        quads = np.ctypeslib.as_array(m.quads, shape=(Q * 4,)).copy().reshape(Q, 4) if Q else np.zeros((0, 4), np.uint32)
        out = dict(vertices=verts, quads=quads, n_active=int(m.n_active), n_lut2=int(m.n_lut2),
                   n_dropped_quads=int(m.n_dropped_quads), n_iso_samples=int(m.n_iso_samples))
        if precision == 0:
            # dual vertices of patches without an in-volume owner edge (the
            # reference leaves them uninitialised): a boolean per vertex
            out["ownerless"] = (np.ctypeslib.as_array(m.ownerless, shape=(V,)).astype(bool)
                                if V else np.zeros(0, bool))
    finally:
        lib().oracle_free(ctypes.byref(m))
    out["triangles"] = quads_to_triangles(out["quads"])
    return out


def quads_to_triangles(quads):
    """Reference split of a quad into (q0,q1,q2), (q2,q3,q0) (dmc.cu:2039-2045)."""
    q = np.asarray(quads).reshape(-1, 4)
    t = np.empty((q.shape[0] * 2, 3), np.uint32)
    t[0::2] = q[:, [0, 1, 2]]
    t[1::2] = q[:, [2, 3, 0]]
    return t
