"""Allocation failures injected on the host: DMC_OPT_FAIL_ALLOCS makes the
context's next device allocations fail as on a device out of memory.  Each
form returns DMC_ERR_OOM, and the context's next call gives the oracle's
mesh: nothing carved from a released buffer is used again (the batch
layout and its captured graph are re-made).  Nothing here faults or stalls
the GPU: the failures happen before any launch that would use the memory."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

OOM = 2


def _vols(n, seed, lo, hi):
    from framework_gb300 import fields
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        dims = tuple(int(d) for d in rng.integers(lo, hi, 3))
        t = fields.gyroid(dims, 0.2 + 0.02 * i, seed=seed + i).cuda()
        out.append(dict(volume=t.contiguous(), iso=float(rng.uniform(-0.3, 0.3))))
    return out


def _check_batch(ex, vols, mode):
    import torch
    V, Q, _ = ex.extract_batch(vols)              # count only
    v = torch.empty((max(V, 1), 3), device="cuda")
    q = torch.empty((max(Q, 1), 4), dtype=torch.int32, device="cuda")
    if mode == "sync":
        nv, nq, res = ex.extract_batch(vols, v, q)
    else:
        ex.extract_batch(vols, v, q, mode=mode)
        nv, nq, res = ex.batch_wait()
    assert (nv, nq) == (V, Q)
    for d, r in zip(vols, res):
        want = oracle.extract(d["volume"].cpu().numpy(), iso=d["iso"])
        vo, n_v, qo, n_q = (int(x) for x in r)
        assert np.array_equal(v[vo:vo + n_v].cpu().numpy().view(np.uint32), want["vertices"].view(np.uint32))
        assert np.array_equal(q[qo:qo + n_q].cpu().numpy().view(np.uint32), want["quads"])


@pytest.mark.parametrize("mode", ["sync", "graph"])
def test_batch_recovers_from_allocation_failure(mode):
    import framework_gb300 as fg
    # the big batch's masks and segments (~60 MB) outgrow the scratch's
    # headroom (1/8 of a scratch that the fixed per-warp spill region keeps
    # above 100 MB), so its layout needs a new scratch
    small, big = _vols(3, 1, 20, 50), _vols(2, 2, 300, 384)
    with fg.Extractor(0, algo="brick") as ex:
        _check_batch(ex, small, mode)                 # scratch, layout (and graph) for the small batch
        ex.set_option(fg.OPT_FAIL_ALLOCS, 1)
        with pytest.raises(fg.DMCError) as e:
            ex.extract_batch(big)                     # a larger layout: the old scratch goes, the new one fails
        assert e.value.status == OOM
        assert e.value.cuda_error.startswith("cudaErrorMemoryAllocation")
        _check_batch(ex, big, mode)                   # carved again on a new scratch
        _check_batch(ex, small, mode)


def test_run_recovers_from_allocation_failure():
    import framework_gb300 as fg
    from framework_gb300 import fields
    host = fields.as_u16_numpy(fields.value_noise_u16((96, 80, 72), base_period=12, seed=6))

    def check(m, iso):
        want = oracle.extract(host, iso=iso)
        assert np.array_equal(m.vertices.view(np.uint32), want["vertices"].view(np.uint32))
        assert np.array_equal(m.quads, want["quads"]) and np.array_equal(m.triangles, want["triangles"])

    with fg.Extractor(0) as ex:
        ex.set_option(fg.OPT_FAIL_ALLOCS, 1)
        with pytest.raises(fg.DMCError) as e:
            ex.run(host, iso=32768.0)                 # the volume's device copy
        assert e.value.status == OOM
        check(ex.run(host, iso=32768.0, triangles=True), 32768.0)
    with fg.Extractor(0) as ex:
        check(ex.run(host, iso=4000.0, triangles=True), 4000.0)   # a small mesh sizes the output buffers
        ex.set_option(fg.OPT_FAIL_ALLOCS, 1)
        with pytest.raises(fg.DMCError) as e:
            ex.run(host, iso=32768.0, triangles=True)  # a larger mesh: the output buffers cannot grow
        assert e.value.status == OOM
        check(ex.run(host, iso=32768.0, triangles=True), 32768.0)
    with fg.Extractor(0) as ex:
        with pytest.raises(fg.DMCError):
            ex.set_option(fg.OPT_FAIL_ALLOCS, -1)
