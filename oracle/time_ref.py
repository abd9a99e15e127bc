#!/usr/bin/env python3
"""Time the reference extractor itself on the GPU host (measurement recipe).

Runs the reference's own dmc::run_dmc (DMC_CUDA/DMC_CUDA/src/dmc.cu:2069-2208),
built by build_ref.py from the staged, unmodified sources, on the benchmark
volumes it can run: C1 (64^3 sphere) and C2 (512^3 blobs), both screened like
the fixtures (no sample at the isovalue, fewer than 4.19 M active cells).  The
1024^3 uint16 volume fails both screens (55,132 samples at the isovalue,
23.5 M active cells), so it is not run.  run_dmc takes host memory in and out
and allocates, copies and synchronises per call; the time is its wall time,
median of the timed calls after one warm-up call, per build.  Prints one JSON
line.  Test infrastructure: never part of the library.
"""
import ctypes
import json
import os
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build_ref  # noqa: E402
import oracle  # noqa: E402


def volumes():
    """(name, volume, iso).  The 512^3 blobs hold samples equal to 0.5, so
    they are timed at the next float above it: the same surface to the eye,
    and no sample at the isovalue."""
    from framework_gb300 import fields
    yield "sphere64", fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).numpy(), 0.0
    yield "blobs512", fields.gaussian_blobs((512, 512, 512)).numpy(), float(np.nextafter(np.float32(0.5), np.float32(1)))


def run(build, name, vol, iso, reps):
    L = ctypes.CDLL(build_ref.build(build))
    L.dmcref_run.restype = ctypes.c_int
    L.dmcref_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_uint,
                             ctypes.POINTER(ctypes.POINTER(ctypes.c_float)), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.POINTER(ctypes.c_uint)), ctypes.POINTER(ctypes.c_uint64)]
    L.dmcref_free.argtypes = [ctypes.c_void_p]
    L.dmcref_setup()
    nz, ny, nx = vol.shape
    dims = (ctypes.c_uint * 3)(nx, ny, nz)
    mn = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
    mx = (ctypes.c_float * 3)(nx - 1.0, ny - 1.0, nz - 1.0)
    times, V, T = [], 0, 0
    for i in range(reps + 1):
        pv, pt = ctypes.POINTER(ctypes.c_float)(), ctypes.POINTER(ctypes.c_uint)()
        nv, nt = ctypes.c_uint64(), ctypes.c_uint64()
        t0 = time.perf_counter()
        rc = L.dmcref_run(vol.ctypes.data, dims, mn, mx, ctypes.c_float(iso), 0, ctypes.byref(pv), ctypes.byref(nv),
                          ctypes.byref(pt), ctypes.byref(nt))
        dt = time.perf_counter() - t0
        assert rc == 0
        L.dmcref_free(pv)
        L.dmcref_free(pt)
        V, T = nv.value, nt.value
        if i:
            times.append(dt)
    L.dmcref_cleanup()
    ms = 1e3 * statistics.median(times)
    return {"build": build, "volume": name, "ms": round(ms, 3), "gvox_per_s": round(vol.size / (ms * 1e-3) / 1e9, 3),
            "vertices": V, "triangles": T, "calls": reps}


def main():
    out = []
    for name, vol, iso in volumes():
        vol = np.ascontiguousarray(vol, np.float32)
        if np.any(vol == np.float32(iso)):
            out.append({"volume": name, "skipped": "a sample equals the isovalue"})
            continue
        if oracle.extract(vol, iso=iso)["n_active"] >= 4_000_000:
            out.append({"volume": name, "skipped": "too many active cells"})
            continue
        for build in ("debug", "release"):
            out.append(dict(run(build, name, vol, iso, 3 if vol.size > 1 << 24 else 10), iso=iso))
    print(json.dumps({"reference_run_dmc": out}))


if __name__ == "__main__":
    main()
