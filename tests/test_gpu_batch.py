"""Batched extraction (``dmc_extract_batch``): every volume's slice of a
batch must be bit-identical to the same volume extracted alone, for mixed
dtypes and shapes, in the synchronous, asynchronous and graph modes."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _mixed_batch(seed=0, count=12):
    """Mixed f32/u16 volumes of uneven shapes, some thin, one without cells."""
    torch = _torch()
    from framework_gb300 import fields
    rng = np.random.default_rng(seed)
    vols = []
    for i in range(count):
        if i == 3:
            shape = (1, 7, 9)                       # no cells
        elif i % 4 == 1:
            shape = (int(rng.integers(2, 6)), int(rng.integers(20, 140)), int(rng.integers(2, 6)))
        else:
            shape = tuple(int(s) for s in rng.integers(4, 90, 3))
        if i % 3 == 2:
            arr = rng.integers(0, 6, shape).astype(np.uint16)
            iso = 2.5 if i % 2 else 3.0
            t = torch.from_numpy(arr.view(np.int16)).cuda()
        else:
            arr = fields.gyroid(shape[::-1], 0.1 + 0.1 * (i % 3), seed=seed + i).numpy()
            assert arr.shape == shape
            iso = float(rng.normal() * 0.1)
            t = torch.from_numpy(arr).cuda()
        mn = tuple(float(x) for x in rng.normal(size=3))
        mx = tuple(mn[k] + float(rng.uniform(0.5, 3.0)) for k in range(3))
        vols.append(dict(volume=t, iso=iso, xyz_min=mn, xyz_max=mx, host=arr))
    return vols


def _alone(ex, d):
    torch = _torch()
    mn, mx = d.get("xyz_min"), d.get("xyz_max")
    nv, nq = ex.extract_device(d["volume"], mn, mx, d["iso"])
    v = torch.empty((max(nv, 1), 3), dtype=torch.float32, device="cuda")
    q = torch.empty((max(nq, 1), 4), dtype=torch.int32, device="cuda")
    t = torch.empty((max(2 * nq, 1), 3), dtype=torch.int32, device="cuda")
    ex.extract_device(d["volume"], mn, mx, d["iso"], v, q, t)
    torch.cuda.synchronize()
    return v[:nv].cpu().numpy(), q[:nq].cpu().numpy(), t[:2 * nq].cpu().numpy()


def _buffers(nv, nq, tris=True):
    torch = _torch()
    v = torch.full((max(nv, 1), 3), float("nan"), dtype=torch.float32, device="cuda")
    q = torch.full((max(nq, 1), 4), -1, dtype=torch.int32, device="cuda")
    t = torch.full((max(2 * nq, 1), 3), -1, dtype=torch.int32, device="cuda") if tris else None
    return v, q, t


def _check_slices(vols, res, v, q, t, alone):
    v, q = v.cpu().numpy(), q.cpu().numpy()
    t = t.cpu().numpy() if t is not None else None
    off_v = off_q = 0
    for i, d in enumerate(vols):
        vo, nv, qo, nq = [int(x) for x in res[i]]
        av, aq, at = alone[i]
        assert (vo, qo) == (off_v, off_q), "volume %d offsets" % i
        assert (nv, nq) == (len(av), len(aq)), "volume %d counts" % i
        assert np.array_equal(v[vo:vo + nv].view(np.uint32), av.view(np.uint32)), "volume %d vertices" % i
        assert np.array_equal(q[qo:qo + nq], aq), "volume %d quads" % i
        if t is not None:
            assert np.array_equal(t[2 * qo:2 * (qo + nq)], at), "volume %d triangles" % i
        off_v += nv
        off_q += nq


@pytest.fixture(scope="module")
def batch_case(extractor):
    vols = _mixed_batch(7)
    alone = [_alone(extractor, d) for d in vols]
    return vols, alone


def test_batch_sync_matches_single(extractor, batch_case):
    vols, alone = batch_case
    NV = sum(len(a[0]) for a in alone)
    NQ = sum(len(a[1]) for a in alone)
    v, q, t = _buffers(NV, NQ)
    nv, nq, res = extractor.extract_batch(vols, v, q, t)
    assert (nv, nq) == (NV, NQ)
    _check_slices(vols, res, v, q, t, alone)


def test_batch_against_oracle(extractor, batch_case):
    vols, _ = batch_case
    small = vols[:6]
    nv, nq, res0 = extractor.extract_batch(small)     # count only
    v, q, t = _buffers(nv, nq)
    nv, nq, res = extractor.extract_batch(small, v, q, t)
    assert np.array_equal(res, res0)
    vh, qh = v.cpu().numpy(), q.cpu().numpy()
    for i, d in enumerate(small):
        vo, n_v, qo, n_q = [int(x) for x in res[i]]
        ref = oracle.extract(d["host"], d["xyz_min"], d["xyz_max"], d["iso"])
        assert np.array_equal(vh[vo:vo + n_v].view(np.uint32), ref["vertices"].view(np.uint32))
        assert np.array_equal(qh[qo:qo + n_q].astype(np.uint32), ref["quads"])


@pytest.mark.parametrize("mode", ["async", "graph"])
def test_batch_async_modes(extractor, batch_case, mode):
    torch = _torch()
    vols, alone = batch_case
    NV = sum(len(a[0]) for a in alone)
    NQ = sum(len(a[1]) for a in alone)
    v, q, t = _buffers(NV + 100, NQ + 100)
    dres = torch.zeros((len(vols), 4), dtype=torch.int64, device="cuda")
    for rep in range(3):   # the graph is captured once and replayed
        v.fill_(float("nan"))
        assert extractor.extract_batch(vols, v, q, t, results=dres, mode=mode) is None
        nv, nq, res = extractor.batch_wait()
        assert (nv, nq) == (NV, NQ)
        _check_slices(vols, res, v, q, t, alone)
        assert np.array_equal(dres.cpu().numpy().astype(np.uint64), res)


def _total(alone):
    return sum(len(a[0]) for a in alone), sum(len(a[1]) for a in alone)


def test_graph_replays_other_batches(extractor, batch_case):
    """One captured graph serves batches of other sizes and shapes."""
    vols, alone = batch_case
    v, q, t = _buffers(*_total(alone))
    n = len(vols)
    for k, idx in enumerate((range(n), range(2, 7), list(range(n))[::-1][:9], [0], range(n))):
        sub = [vols[i] for i in idx]
        if k == 2:
            v, q, t = _buffers(*_total(alone))      # other output buffers: patched into the graph
        tt = None if k == 3 else t
        extractor.extract_batch(sub, v, q, tt, mode="graph")
        nv, nq, res = extractor.batch_wait()
        _check_slices(sub, res, v, q, tt, [alone[i] for i in idx])


def test_batch_overflow(extractor, batch_case):
    from framework_gb300 import DMCError
    vols, alone = batch_case
    NV = sum(len(a[0]) for a in alone)
    NQ = sum(len(a[1]) for a in alone)
    v, q, t = _buffers(NV - 1, NQ)
    with pytest.raises(DMCError) as e:
        extractor.extract_batch(vols, v, q, t)
    assert e.value.status == 3 and e.value.counts == (NV, NQ)
    # asynchronous: checked on the device, reported by the wait
    extractor.extract_batch(vols, v, q, t, mode="async")
    with pytest.raises(DMCError) as e:
        extractor.batch_wait()
    assert e.value.status == 3 and e.value.counts == (NV, NQ)
    # the context is usable afterwards
    v, q, t = _buffers(NV, NQ)
    nv, nq, res = extractor.extract_batch(vols, v, q, t)
    _check_slices(vols, res, v, q, t, alone)


def test_batch_busy(extractor, batch_case):
    from framework_gb300 import DMCError
    vols, alone = batch_case
    v, q, t = _buffers(*_total(alone))
    extractor.extract_batch(vols, v, q, t, mode="async")
    with pytest.raises(DMCError) as e:
        extractor.extract_batch(vols, v, q, t, mode="async")
    assert e.value.status == 1
    with pytest.raises(DMCError) as e:
        extractor.extract_device(vols[0]["volume"], vols[0]["xyz_min"], vols[0]["xyz_max"], vols[0]["iso"])
    assert e.value.status == 1
    nv, nq, res = extractor.batch_wait()
    _check_slices(vols, res, v, q, t, alone)
    with pytest.raises(DMCError):
        extractor.batch_wait()


@pytest.mark.parametrize("planes", [1, 3, 4, 16, 64])
def test_brick_planes_option(extractor, batch_case, planes):
    import framework_gb300 as fg
    vols, alone = batch_case
    v, q, t = _buffers(*_total(alone))
    extractor.set_option(fg.OPT_BRICK_PLANES, planes)
    try:
        nv, nq, res = extractor.extract_batch(vols, v, q, t)
    finally:
        extractor.set_option(fg.OPT_BRICK_PLANES, 0)
    _check_slices(vols, res, v, q, t, alone)


def test_uneven_gyroid_batch(extractor):
    """A smaller instance of the uneven gyroid workload (dims 16..96)."""
    torch = _torch()
    from framework_gb300 import fields
    specs = fields.uneven_batch_specs(count=24, lo=16, hi=96, seed=3)
    vols = []
    for sp in specs:
        t = fields.gyroid(sp["dims"], sp["freq"], seed=sp["seed"]).cuda()
        vols.append(dict(volume=t, iso=sp["iso"]))
    alone = [_alone(extractor, d) for d in vols]
    NV = sum(len(a[0]) for a in alone)
    NQ = sum(len(a[1]) for a in alone)
    v, q, t = _buffers(NV, NQ)
    nv, nq, res = extractor.extract_batch(vols, v, q, t)
    _check_slices(vols, res, v, q, t, alone)


def test_graph_after_layout_growth():
    """Growing batches in graph mode on a fresh context: each growth re-carves
    the scratch layout (often inside the same allocation); the graph must be
    captured again and every batch stay exact."""
    import framework_gb300 as fg
    vols = _mixed_batch(21, count=14)
    with fg.Extractor(0) as ex:
        alone = [_alone(ex, d) for d in vols]
        v, q, t = _buffers(*_total(alone))
        for k in (1, 2, 4, 7, 14, 3):
            ex.extract_batch(vols[:k], v, q, t, mode="graph")
            nv, nq, res = ex.batch_wait()
            _check_slices(vols[:k], res, v, q, t, alone[:k])


def test_default_stream_ordering(extractor, batch_case):
    """A volume written by torch on its current stream just before an
    asynchronous batch is seen complete by the batch."""
    torch = _torch()
    vols, alone = batch_case
    v, q, t = _buffers(*_total(alone))
    scratch = [dict(d, volume=torch.empty_like(d["volume"])) for d in vols]
    for rep in range(2):
        for s, d in zip(scratch, vols):
            s["volume"].zero_()
            s["volume"].copy_(d["volume"])
        extractor.extract_batch(scratch, v, q, t, mode="graph" if rep else "async")
        nv, nq, res = extractor.batch_wait()
        _check_slices(vols, res, v, q, t, alone)


def test_autotune_persists(extractor, batch_case, tmp_path):
    from framework_gb300 import autotune
    vols, alone = batch_case
    v, q, t = _buffers(*_total(alone))
    cache = str(tmp_path / "tune.json")
    r1 = autotune.tune(extractor, vols, v, q, t, candidates=(0, 4, 16), reps=1, cache=cache)
    assert not r1["cached"] and r1["planes"] in (0, 4, 16) and set(r1["ms"]) == {"0", "4", "16"}
    r2 = autotune.tune(extractor, vols, v, q, t, candidates=(0, 4, 16), reps=1, cache=cache)
    assert r2["cached"] and r2["planes"] == r1["planes"]
    # the tuned option leaves the meshes unchanged
    nv, nq, res = extractor.extract_batch(vols, v, q, t)
    _check_slices(vols, res, v, q, t, alone)
    import framework_gb300 as fg
    extractor.set_option(fg.OPT_BRICK_PLANES, 0)
