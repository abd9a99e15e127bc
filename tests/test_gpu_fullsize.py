"""Parity at the benchmark sizes: the 64^3 sphere, the 512^3 float32 blobs
and the 1024^3 uint16 value noise, extracted on the GPU and by the CPU oracle
(all host threads), must agree bit for bit; the brick and simple kernel
families must agree with each other on the device as well.  Against the FP64
oracle the topology must be identical and the vertices within the bound of
tests/fp64bound.py (4 ulp of the extent's largest coordinate)."""
import os

import numpy as np
import pytest

import fp64bound
import oracle

pytestmark = pytest.mark.gpu


def _device_mesh(ex, vol, iso, algo):
    import torch
    ex.set_algo(algo)
    try:
        nv, nq = ex.extract_device(vol, iso=iso)
        v = torch.empty((nv, 3), dtype=torch.float32, device="cuda")
        q = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
        ex.extract_device(vol, iso=iso, vertices=v, quads=q)
        torch.cuda.synchronize()
        st = ex.stats()
    finally:
        ex.set_algo("auto")
    return v, q, st


def _full_case(extractor, name):
    import torch
    from framework_gb300 import fields
    if name == "sphere64":
        vol, iso = fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).cuda(), 0.0
        host = vol.cpu().numpy()
    elif name == "blobs512":
        vol, iso = fields.gaussian_blobs((512, 512, 512), device="cuda"), 0.5
        host = vol.cpu().numpy()
    else:
        vol, iso = fields.value_noise_u16((1024, 1024, 1024), device="cuda"), 32768.0
        host = fields.as_u16_numpy(vol)
    torch.cuda.synchronize()
    vb, qb, st = _device_mesh(extractor, vol, iso, "brick")
    vs, qs, _ = _device_mesh(extractor, vol, iso, "simple")
    # brick and simple families agree on the device (bitwise)
    assert torch.equal(vb.view(torch.int32), vs.view(torch.int32))
    assert torch.equal(qb, qs)
    del vs, qs
    oracle.set_threads(os.cpu_count() or 1)
    ref = oracle.extract(host, iso=iso)
    assert vb.shape[0] == len(ref["vertices"]) and qb.shape[0] == len(ref["quads"])
    assert st["n_active_cells"] == ref["n_active"] and st["n_lut2_cells"] == ref["n_lut2"]
    assert st["n_dropped_quads"] == ref["n_dropped_quads"]
    gv = vb.cpu().numpy()
    assert np.array_equal(gv.view(np.uint32), ref["vertices"].view(np.uint32))
    del gv
    assert np.array_equal(qb.cpu().numpy().view(np.uint32), ref["quads"])
    V, Q = len(ref["vertices"]), len(ref["quads"])
    del ref
    ref64 = oracle.extract(host, iso=iso, precision=1)
    assert np.array_equal(qb.cpu().numpy().view(np.uint32), ref64["quads"])      # same topology
    worst, ulps, vox = fp64bound.check(vb.cpu().numpy(), ref64["vertices"], host.shape[::-1])
    print("%s: FP32 vs FP64 max |d| %.3g = %.2f ulp(M) = %.3g voxel" % (name, worst, ulps, vox))
    return V, Q


def test_sphere64_full_size(extractor):
    V, Q = _full_case(extractor, "sphere64")
    assert V > 10000 and Q > 5000


def test_blobs512_full_size(extractor):
    V, Q = _full_case(extractor, "blobs512")
    assert V > 100000 and Q > 50000


def test_noise1024_full_size(extractor):
    V, Q = _full_case(extractor, "noise1024")
    assert V > 40_000_000 and Q > 20_000_000
