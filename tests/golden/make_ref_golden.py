#!/usr/bin/env python3
"""Golden fixtures made by the reference extractor itself: tests/golden/ref_*.npz.

Runs the reference's own dmc::run_dmc (DMC_CUDA/DMC_CUDA/src/dmc.cu:2069-2208),
built from its unmodified sources by oracle/build_ref.py, on small seeded
volumes, and stores each input with the reference's vertices and triangles.
It needs a GPU and the staged sources (oracle/_ref/src, from
`DMC_REFERENCE_DIR=... python oracle/build_ref.py --stage`).

Every input is screened first, because the reference misbehaves outside
these limits (those are the inputs the fixtures stay away from):
  * no sample equal to the isovalue: its bipolar test (dmc.cu:1101-1106) then
    accepts edges whose cells are inactive, and the quad walk reads an
    invalid index map entry (out-of-bounds device reads);
  * fewer than 4.19 M active cells: its grid fold (dmc.cu:2116-2120) drops
    blocks when an odd block count is halved.

Three builds are run, each in its own process: "debug" (-G, the reference's
shipped configuration), "release" (-O3, FMA contraction allowed) and "nofma"
(-O3 -fmad=false).  Output per case: volume, iso, xyz_min, xyz_max, and
vertices_<build>, triangles_<build>.

Usage (on the GPU host): python tests/golden/make_ref_golden.py [out_dir]
"""
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

BUILDS = ("debug", "release", "nofma")
MAX_ACTIVE = 4_000_000


def cases():
    """(name, float32 volume [z, y, x], iso, xyz_min, xyz_max)."""
    from framework_gb300 import fields
    yield ("sphere64", fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).numpy(), 0.0,
           (0.0, 0.0, 0.0), (63.0, 63.0, 63.0))
    for name in ("sphere24", "blobs_noncubic", "gyroid", "checker"):
        g = np.load(os.path.join(HERE, name + ".npz"))
        yield ("g_" + name, g["volume"].astype(np.float32), float(g["iso"]), tuple(g["xyz_min"].tolist()),
               tuple(g["xyz_max"].tolist()))
    g = np.load(os.path.join(HERE, "noise_u16.npz"))
    v = g["volume"].astype(np.float32)
    nz, ny, nx = v.shape
    yield "g_noise_u16_half", v, 32767.5, (0.0, 0.0, 0.0), (nx - 1.0, ny - 1.0, nz - 1.0)
    rng = np.random.default_rng(77)
    yield ("random_ambiguous", rng.random((16, 18, 20), dtype=np.float32), 0.5, (0.0, 0.0, 0.0),
           (19.0, 17.0, 15.0))
    yield ("random_offset_extent", rng.random((19, 23, 17), dtype=np.float32), 0.3, (-7.5, 2.25, 100.0),
           (3.0, 9.0, 130.5))
    b = fields.gaussian_blobs((40, 36, 30), count=5, sigma=(4.0, 8.0), seed=3).numpy()
    yield "blobs40", b, 0.5, (0.0, 0.0, 0.0), (39.0, 35.0, 29.0)


def screen(vol, iso):
    import oracle
    if np.any(vol == np.float32(iso)):
        raise ValueError("a sample equals the isovalue")
    r = oracle.extract(vol, iso=iso)
    if r["n_active"] >= MAX_ACTIVE:
        raise ValueError("too many active cells for the reference's grid fold")
    return r["n_active"]


def run_build(build, inputs, out):
    """Child process: load one build of the reference and run every case."""
    from oracle import build_ref
    L = ctypes.CDLL(build_ref.build(build))
    L.dmcref_run.restype = ctypes.c_int
    L.dmcref_run.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_float),
                             ctypes.POINTER(ctypes.c_float), ctypes.c_float, ctypes.c_uint,
                             ctypes.POINTER(ctypes.POINTER(ctypes.c_float)), ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.POINTER(ctypes.c_uint)), ctypes.POINTER(ctypes.c_uint64)]
    L.dmcref_free.argtypes = [ctypes.c_void_p]
    L.dmcref_setup()
    data = np.load(inputs)
    res = {}
    for name in data["names"]:
        name = str(name)
        vol = np.ascontiguousarray(data["vol_" + name])
        nz, ny, nx = vol.shape
        dims = (ctypes.c_uint * 3)(nx, ny, nz)
        mn = (ctypes.c_float * 3)(*data["mn_" + name].tolist())
        mx = (ctypes.c_float * 3)(*data["mx_" + name].tolist())
        pv, pt = ctypes.POINTER(ctypes.c_float)(), ctypes.POINTER(ctypes.c_uint)()
        nv, nt = ctypes.c_uint64(), ctypes.c_uint64()
        rc = L.dmcref_run(vol.ctypes.data, dims, mn, mx, ctypes.c_float(float(data["iso_" + name])), 0,
                          ctypes.byref(pv), ctypes.byref(nv), ctypes.byref(pt), ctypes.byref(nt))
        assert rc == 0, rc
        V, T = nv.value, nt.value
        res["v_" + name] = np.ctypeslib.as_array(pv, shape=(max(V, 1) * 3,))[:V * 3].copy().reshape(V, 3)
        res["t_" + name] = np.ctypeslib.as_array(pt, shape=(max(T, 1) * 3,))[:T * 3].copy().reshape(T, 3)
        L.dmcref_free(pv)
        L.dmcref_free(pt)
    L.dmcref_cleanup()
    np.savez(out, **res)


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    todo = []
    for name, vol, iso, mn, mx in cases():
        n_active = screen(vol, iso)
        todo.append((name, vol, iso, mn, mx))
        print("%-22s %-14s iso %-8g active %d" % (name, vol.shape, iso, n_active))
    with tempfile.TemporaryDirectory() as tmp:
        inputs = os.path.join(tmp, "inputs.npz")
        arrays = {"names": np.array([c[0] for c in todo])}
        for name, vol, iso, mn, mx in todo:
            arrays["vol_" + name] = vol
            arrays["iso_" + name] = np.float32(iso)
            arrays["mn_" + name] = np.array(mn, np.float32)
            arrays["mx_" + name] = np.array(mx, np.float32)
        np.savez(inputs, **arrays)
        outs = {}
        for b in BUILDS:
            out = os.path.join(tmp, b + ".npz")
            subprocess.check_call([sys.executable, os.path.abspath(__file__), "--run", b, inputs, out], cwd=ROOT)
            outs[b] = np.load(out)
        for name, vol, iso, mn, mx in todo:
            fx = dict(volume=vol, iso=np.float32(iso), xyz_min=np.array(mn, np.float32),
                      xyz_max=np.array(mx, np.float32))
            for b in BUILDS:
                fx["vertices_" + b] = outs[b]["v_" + name]
                fx["triangles_" + b] = outs[b]["t_" + name]
            np.savez_compressed(os.path.join(out_dir, "ref_" + name + ".npz"), **fx)
            print("%-22s V=%d T=%d" % (name, len(fx["vertices_debug"]), len(fx["triangles_debug"])))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--run":
        run_build(sys.argv[2], sys.argv[3], sys.argv[4])
    else:
        main(sys.argv[1] if len(sys.argv) > 1 else HERE)
