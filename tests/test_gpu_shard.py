"""Sharded extraction of one volume (dmc_shard_count / dmc_shard_emit): the
parts of all ranks, concatenated in rank order, equal the unsharded mesh bit
for bit.  The ranks run one after another on one GPU, each on its own
context holding only its own point planes; the exchange of totals is the
exclusive scan that the all-gather feeds (the collective itself runs on CPU
ranks in test_multirank_cpu.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(kind):
    from framework_gb300 import fields
    if kind == "u16":
        return fields.value_noise_u16((150, 70, 261), base_period=16, seed=12).cuda(), 32768.0
    if kind == "f32":
        return fields.gaussian_blobs((140, 90, 300), seed=5, device="cuda"), 0.5
    return fields.gyroid((40, 50, 97), 0.3, seed=3).cuda(), 0.1


def _whole(ex, vol, iso, mn, mx):
    import torch
    nv, nq = ex.extract_device(vol, mn, mx, iso)
    v = torch.empty((nv, 3), device="cuda")
    q = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
    t = torch.empty((2 * nq, 3), dtype=torch.int32, device="cuda")
    ex.extract_device(vol, mn, mx, iso, v, q, t)
    return v.cpu().numpy(), q.cpu().numpy(), t.cpu().numpy()


def _sharded(vol, iso, mn, mx, ranges):
    import torch
    import framework_gb300 as fg
    from framework_gb300 import shard
    nz = vol.shape[0]
    exs = [fg.Extractor(0) for _ in ranges]
    try:
        locals_, totals = [], []
        for ex, (zb, ze) in zip(exs, ranges):
            p0, p1 = shard.point_planes(nz, zb, ze)
            local = vol[p0:p1].clone()                   # the rank's own copy of its planes
            locals_.append(local)
            totals.append(ex.shard_count(local, nz, zb, ze, mn, mx, iso))
        parts = []
        for r, ex in enumerate(exs):
            nv, nq = totals[r]
            voff, _ = shard.exclusive_offsets(totals, r)
            v = torch.full((max(nv, 1), 3), float("nan"), device="cuda")
            q = torch.full((max(nq, 1), 4), -1, dtype=torch.int32, device="cuda")
            t = torch.full((max(2 * nq, 1), 3), -1, dtype=torch.int32, device="cuda")
            ex.shard_emit(voff, v, q, t)
            parts.append((v[:nv].cpu().numpy(), q[:nq].cpu().numpy(), t[:2 * nq].cpu().numpy()))
        return totals, parts
    finally:
        for ex in exs:
            ex.close()


@pytest.mark.parametrize("kind,split", [("u16", 2), ("u16", 5), ("f32", 3), ("f32", "odd"), ("gyr", 4), ("u16", "odd")])
def test_shards_equal_whole(extractor, kind, split):
    from framework_gb300 import shard
    vol, iso = _case(kind)
    cz = vol.shape[0] - 1
    mn, mx = (-1.0, 0.5, 2.0), (3.0, 4.0, 11.0)
    want = _whole(extractor, vol, iso, mn, mx)
    if split == "odd":
        # one-plane shards and cuts on no power of two
        cuts = [0, 1, 37, 38, 100, 211, cz]
        ranges = list(zip(cuts[:-1], cuts[1:]))
    else:
        ranges = shard.shard_ranges(cz, split, align=8 if kind == "gyr" else 32)
    totals, parts = _sharded(vol, iso, mn, mx, ranges)
    assert sum(t[0] for t in totals) == len(want[0]) and sum(t[1] for t in totals) == len(want[1])
    got_v = np.concatenate([p[0] for p in parts])
    got_q = np.concatenate([p[1] for p in parts])
    got_t = np.concatenate([p[2] for p in parts])
    assert np.array_equal(got_v.view(np.uint32), want[0].view(np.uint32))
    assert np.array_equal(got_q, want[1]) and np.array_equal(got_t, want[2])


def test_shard_errors(extractor):
    import torch
    import framework_gb300 as fg
    vol, iso = _case("gyr")
    nz = vol.shape[0]
    with pytest.raises(fg.DMCError) as e:          # wrong local plane count
        extractor.shard_count(vol[0:10].contiguous(), nz, 0, 20, None, None, iso)
    assert e.value.status == 1
    with pytest.raises(fg.DMCError) as e:          # empty range
        extractor.shard_count(vol[0:3].contiguous(), nz, 5, 5, None, None, iso)
    assert e.value.status == 1
    v = torch.empty((4, 3), device="cuda")
    q = torch.empty((4, 4), dtype=torch.int32, device="cuda")
    with fg.Extractor(0) as fresh:
        with pytest.raises(fg.DMCError) as e:      # emit without a count on this context
            fresh.shard_emit(0, v, q)
    assert e.value.status == 1
    nv, nq = extractor.shard_count(vol[0:nz].contiguous(), nz, 0, nz - 1, None, None, iso)
    with pytest.raises(fg.DMCError) as e:          # too small buffers
        extractor.shard_emit(0, v, q)
    assert e.value.status == 3
    # another extraction between the phases replaces the count's plan
    extractor.shard_count(vol[0:nz].contiguous(), nz, 0, nz - 1, None, None, iso)
    extractor.extract_device(vol, iso=iso)
    vb = torch.empty((nv, 3), device="cuda")
    qb = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
    with pytest.raises(fg.DMCError) as e:
        extractor.shard_emit(0, vb, qb)
    assert e.value.status == 1
    # a whole-volume shard is the whole mesh
    extractor.shard_count(vol[0:nz].contiguous(), nz, 0, nz - 1, None, None, iso)
    extractor.shard_emit(0, vb, qb)
    wv, wq, _ = _whole(extractor, vol, iso, None, None)
    assert np.array_equal(vb.cpu().numpy().view(np.uint32), wv.view(np.uint32))
    assert np.array_equal(qb.cpu().numpy(), wq)
