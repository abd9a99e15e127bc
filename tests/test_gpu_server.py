"""Serving loop (``dmc_server_*``): every request's mesh, served in a mix of
concurrent requests, batched and overlapped on the device, is bit-identical
to the same (volume, isovalue) extracted alone with dmc_extract_device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pool(seed=11):
    import torch
    from framework_gb300 import fields
    rng = np.random.default_rng(seed)
    vols = []
    for i in range(8):
        dims = tuple(int(d) for d in rng.integers(12, 120, 3))
        if i == 2:
            dims = (130, 5, 40)                       # ragged, wider than one brick
        if i % 3 == 1:
            t = fields.value_noise_u16(dims, base_period=16, seed=20 + i).cuda()
            host = fields.as_u16_numpy(t).astype(np.float64)
        elif i % 3 == 2:
            t = fields.gaussian_blobs(dims, seed=30 + i, device="cuda")
            host = t.cpu().numpy().astype(np.float64)
        else:
            t = fields.gyroid(dims, 0.15 + 0.05 * i, seed=40 + i).cuda()
            host = t.cpu().numpy().astype(np.float64)
        lo, hi = np.percentile(host, [5, 95])
        mn = tuple(float(x) for x in rng.normal(size=3))
        mx = tuple(mn[k] + float(rng.uniform(1.0, 4.0)) for k in range(3))
        vols.append(dict(volume=t.contiguous(), lo=float(lo), hi=float(hi), xyz_min=mn, xyz_max=mx))
    torch.cuda.synchronize()
    return vols


def _requests(vols, n, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        v = int(rng.integers(0, len(vols)))
        iso = float(rng.uniform(vols[v]["lo"], vols[v]["hi"]))
        if str(vols[v]["volume"].dtype) == "torch.int16":
            iso = float(np.floor(iso)) + (0.5 if rng.random() < 0.5 else 0.0)   # also exact integers
        out.append((v, iso))
    return out


def _alone(ex, d, iso):
    import torch
    nv, nq = ex.extract_device(d["volume"], d["xyz_min"], d["xyz_max"], iso)
    v = torch.empty((max(nv, 1), 3), dtype=torch.float32, device="cuda")
    q = torch.empty((max(nq, 1), 4), dtype=torch.int32, device="cuda")
    t = torch.empty((max(2 * nq, 1), 3), dtype=torch.int32, device="cuda")
    ex.extract_device(d["volume"], d["xyz_min"], d["xyz_max"], iso, v, q, t)
    torch.cuda.synchronize()
    return v[:nv].cpu().numpy(), q[:nq].cpu().numpy().view(np.uint32), t[:2 * nq].cpu().numpy().view(np.uint32)


@pytest.fixture(scope="module")
def pool_case(extractor):
    vols = _pool()
    reqs = _requests(vols, 48)
    alone = {}
    for v, iso in reqs:
        if (v, iso) not in alone:
            alone[(v, iso)] = _alone(extractor, vols[v], iso)
    return vols, reqs, alone


def _check(srv, res, want):
    assert res["status"] == 0
    got = srv.fetch(res)
    assert got[0].shape == want[0].shape and got[1].shape == want[1].shape
    assert np.array_equal(got[0].view(np.uint32), want[0].view(np.uint32))
    assert np.array_equal(got[1], want[1])
    if got[2] is not None:
        assert np.array_equal(got[2], want[2])
    assert res["t_submit"] <= res["t_start"] <= res["t_done"]


def _serve(srv, vols, reqs, alone, release_order=None, stream=False):
    """Submits all requests at once (they overlap), then checks each result.
    stream=True releases each result right after its check, so a small arena
    can admit the next requests; otherwise results are released at the end,
    in release_order."""
    ids = [srv.add_volume(d["volume"], d["xyz_min"], d["xyz_max"]) for d in vols]
    rids = [srv.submit(ids[v], iso) for v, iso in reqs]
    results = []
    for (v, iso), rid in zip(reqs, rids):
        res = srv.wait(rid, timeout=120.0)
        _check(srv, res, alone[(v, iso)])
        results.append(res)
        if stream:
            srv.release(rid)
    if not stream:
        for i in (release_order(len(rids)) if release_order else range(len(rids))):
            srv.release(rids[i])
    return results


def test_served_equals_alone(pool_case):
    import framework_gb300 as fg
    vols, reqs, alone = pool_case
    with fg.Server(0, vertex_arena=1 << 26, quad_arena=1 << 25, lanes=2, max_batch=16, triangles=True) as srv:
        results = _serve(srv, vols, reqs, alone, release_order=lambda n: list(range(n))[::-1])
        st = srv.stats()
    assert st["submitted"] == st["completed"] == len(reqs)
    assert st["batches"] < len(reqs) and st["max_batch_seen"] > 1       # requests were batched
    assert max(r["batch_size"] for r in results) > 1


def test_served_under_arena_pressure(pool_case):
    """An arena that holds only about one worst-case request at a time:
    admission waits for space, results are unchanged."""
    import framework_gb300 as fg
    vols, reqs, alone = pool_case
    cells = max((d["volume"].shape[0] - 1) * (d["volume"].shape[1] - 1) * (d["volume"].shape[2] - 1) for d in vols)
    with fg.Server(0, vertex_arena=7 * cells + 4096, quad_arena=3 * cells + 4096, lanes=2, max_batch=8) as srv:
        _serve(srv, vols, reqs[:20], alone, stream=True)
        st = srv.stats()
    assert st["completed"] == 20
    assert st["arena_peak_vertices"] <= 7 * cells + 4096


def test_plain_mode_equals_alone(pool_case):
    import framework_gb300 as fg
    vols, reqs, alone = pool_case
    with fg.Server(0, vertex_arena=1 << 26, quad_arena=1 << 25, plain=True) as srv:
        results = _serve(srv, vols, reqs[:12], alone)
    assert all(r["batch_size"] == 1 for r in results)


def test_server_errors(pool_case):
    import framework_gb300 as fg
    vols, _, _ = pool_case
    with fg.Server(0, vertex_arena=4096, quad_arena=4096) as srv:
        with pytest.raises(fg.DMCError) as e:
            srv.add_volume(vols[0]["volume"])                         # bound exceeds the arenas
        assert e.value.status == 3
        with pytest.raises(fg.DMCError) as e:
            srv.submit(5, 0.0)                                        # no such volume
        assert e.value.status == 1
        with pytest.raises(fg.DMCError):
            srv.wait(12345, timeout=0.0)
        with pytest.raises(fg.DMCError):
            srv.release(12345)


def test_replay_load_generator(pool_case):
    import framework_gb300 as fg
    vols, reqs, _ = pool_case
    rng = np.random.default_rng(5)
    arrivals = np.cumsum(rng.exponential(1e-3, size=len(reqs)))   # ~1000 requests/s
    with fg.Server(0, vertex_arena=1 << 26, quad_arena=1 << 25) as srv:
        ids = [srv.add_volume(d["volume"], d["xyz_min"], d["xyz_max"]) for d in vols]
        lat, st = srv.replay([ids[v] for v, _ in reqs], [iso for _, iso in reqs], arrivals)
        stats = srv.stats()
    assert (st == 0).all() and (lat > 0).all() and (lat < 30).all()
    assert stats["completed"] == len(reqs)


def test_fetch_into_host_buffers(pool_case):
    """Server.fetch_into copies a result into caller buffers (pinned torch
    tensors, plain numpy arrays) with the same bits as fetch; short buffers
    give OUTPUT_OVERFLOW with the counts."""
    import torch
    import framework_gb300 as fg
    vols, reqs, alone = pool_case
    with fg.Server(0, vertex_arena=1 << 26, quad_arena=1 << 25, triangles=True) as srv:
        ids = [srv.add_volume(d["volume"], d["xyz_min"], d["xyz_max"]) for d in vols]
        for v, iso in reqs[:6]:
            rid = srv.submit(ids[v], iso)
            res = srv.wait(rid, timeout=120.0)
            want = alone[(v, iso)]
            nv, nq = len(want[0]), len(want[1])
            hv = torch.empty((nv + 5, 3), dtype=torch.float32, pin_memory=True)
            hq = torch.empty((nq + 5, 4), dtype=torch.int32, pin_memory=True)
            ht = np.empty((2 * nq + 5, 3), np.uint32)
            assert srv.fetch_into(res, hv, hq, ht) == (nv, nq)
            assert np.array_equal(hv[:nv].numpy().view(np.uint32), want[0].view(np.uint32))
            assert np.array_equal(hq[:nq].numpy().view(np.uint32), want[1])
            assert np.array_equal(ht[:2 * nq], want[2])
            if nq > 1:
                with pytest.raises(fg.DMCError) as e:
                    srv.fetch_into(res, hv, hq[:nq - 1])
                assert e.value.status == 3 and e.value.counts == (nv, nq)
            srv.release(rid)


def test_fetch_into_on_stream(pool_case):
    """fetch_into with a stream only enqueues the copies: a burst of results
    fetched into a ring of pinned buffers, each request released after an
    event on the copy stream, gives every mesh with fetch's bits."""
    import torch
    import framework_gb300 as fg
    vols, reqs, alone = pool_case
    cs = torch.cuda.Stream()
    with fg.Server(0, vertex_arena=1 << 26, quad_arena=1 << 25, triangles=True) as srv:
        ids = [srv.add_volume(d["volume"], d["xyz_min"], d["xyz_max"]) for d in vols]
        vmax = max(len(w[0]) for w in alone.values()) + 1
        qmax = max(len(w[1]) for w in alone.values()) + 1
        bufs = [(torch.empty((vmax, 3), dtype=torch.float32, pin_memory=True),
                 torch.empty((qmax, 4), dtype=torch.int32, pin_memory=True),
                 torch.empty((2 * qmax, 3), dtype=torch.int32, pin_memory=True)) for _ in range(3)]
        rids = [srv.submit(ids[v], iso) for v, iso in reqs]
        pending = []
        for i, (rid, key) in enumerate(zip(rids, reqs)):
            if len(pending) == 3:
                _check_fetched(srv, *pending.pop(0), alone)
            hv, hq, ht = bufs[i % 3]
            res = srv.wait(rid, timeout=120.0)
            n = srv.fetch_into(res, hv, hq, ht, stream=cs)
            ev = torch.cuda.Event()
            ev.record(cs)
            pending.append((rid, key, n, ev, (hv, hq, ht)))
        for p in pending:
            _check_fetched(srv, *p, alone)


def _check_fetched(srv, rid, key, n, ev, bufs, alone):
    ev.synchronize()
    srv.release(rid)
    hv, hq, ht = bufs
    want = alone[key]
    nv, nq = n
    assert (nv, nq) == (len(want[0]), len(want[1]))
    assert np.array_equal(hv[:nv].numpy().view(np.uint32), want[0].view(np.uint32))
    assert np.array_equal(hq[:nq].numpy().view(np.uint32), want[1])
    assert np.array_equal(ht[:2 * nq].numpy().view(np.uint32), want[2])
