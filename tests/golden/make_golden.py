#!/usr/bin/env python3
"""Regenerate the golden fixtures in tests/golden.

Each fixture holds a small seeded input volume, its extraction parameters and
the CPU oracle's output (oracle/dmc_oracle.c, FP32 replica).  The reference
itself cannot run in the build container (it is CUDA-only), so these goldens
pin the oracle's behaviour: tests check the oracle still reproduces them, that
they satisfy mesh invariants, and that the GPU matches them bit for bit.

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from framework_gb300 import fields  # noqa: E402


def cases():
    rng = np.random.default_rng(20240611)
    yield "sphere24", fields.sphere_sdf(24, radius=8.0, noise=0.01, seed=11).numpy(), 0.0, None, None
    v = fields.value_noise_u16((21, 17, 23), base_period=8, seed=12)
    yield "noise_u16", fields.as_u16_numpy(v), 32768.0, None, None
    b = fields.gaussian_blobs((33, 29, 26), count=6, sigma=(3.0, 6.0), seed=13).numpy()
    yield "blobs_noncubic", b, 0.5, (-1.0, -2.0, 0.5), (3.0, 1.0, 4.0)
    yield "gyroid", fields.gyroid((19, 22, 20), 0.6, noise=0.02, seed=14).numpy(), 0.1, (-5.0, -5.0, -5.0), (5.0, 5.0, 5.0)
    # integer-valued field: many samples exactly at the isovalue, many ambiguous faces
    yield "ints_u16", rng.integers(0, 3, (9, 11, 10)).astype(np.uint16), 1.0, None, None
    yield "checker", ((np.indices((7, 8, 9)).sum(0) % 2) * 2 - 1).astype(np.float32), 0.0, None, None


def main():
    for name, vol, iso, mn, mx in cases():
        r = oracle.extract(vol, mn, mx, iso)
        nz, ny, nx = vol.shape
        np.savez_compressed(os.path.join(HERE, name + ".npz"), volume=vol, iso=np.float32(iso),
                            xyz_min=np.array(mn if mn else (0, 0, 0), np.float32),
                            xyz_max=np.array(mx if mx else (nx - 1, ny - 1, nz - 1), np.float32),
                            vertices=r["vertices"], quads=r["quads"],
                            counters=np.array([r["n_active"], r["n_lut2"], r["n_dropped_quads"], r["n_iso_samples"]], np.int64))
        print(name, vol.shape, vol.dtype, "V=%d Q=%d active=%d lut2=%d dropped=%d iso_samples=%d" % (
            len(r["vertices"]), len(r["quads"]), r["n_active"], r["n_lut2"], r["n_dropped_quads"], r["n_iso_samples"]))


if __name__ == "__main__":
    main()
