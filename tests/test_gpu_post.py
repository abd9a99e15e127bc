"""dmc_compact_mesh (opt-in post-processing): keeps exactly the vertices the
quads reference, in order, and renumbers quads and triangles; checked against
a numpy restatement of the same integer work."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mesh(extractor, vol, iso):
    import torch
    nv, nq = extractor.extract_device(vol, iso=iso)
    v = torch.empty((nv, 3), device="cuda")
    q = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
    t = torch.empty((2 * nq, 3), dtype=torch.int32, device="cuda")
    extractor.extract_device(vol, iso=iso, vertices=v, quads=q, triangles=t)
    return v, q, t


@pytest.mark.parametrize("case", ["sphere", "noise"])
def test_compact_matches_numpy(extractor, case):
    from framework_gb300 import fields
    if case == "sphere":
        vol, iso = fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).cuda(), 0.0
    else:
        vol, iso = fields.value_noise_u16((150, 90, 70), base_period=16, seed=5).cuda(), 32768.0
    v, q, t = _mesh(extractor, vol, iso)
    V, Q, T = v.cpu().numpy(), q.cpu().numpy().astype(np.int64), t.cpu().numpy().astype(np.int64)
    used = np.unique(Q)
    out = extractor.compact_mesh(v, q, t)
    assert out.shape[0] == used.size < V.shape[0]
    assert np.array_equal(out.cpu().numpy().view(np.uint32), V[used].view(np.uint32))
    assert np.array_equal(q.cpu().numpy(), np.searchsorted(used, Q))
    assert np.array_equal(t.cpu().numpy(), np.searchsorted(used, T))
    # the same faces, now over the kept vertices
    assert np.array_equal(out.cpu().numpy()[q.cpu().numpy()], V[Q])


def test_compact_errors(extractor):
    import torch
    import framework_gb300 as fg
    v = torch.zeros((10, 3), device="cuda")
    q = torch.tensor([[0, 1, 2, 3], [4, 5, 6, 10]], dtype=torch.int32, device="cuda")   # 10 is out of range
    with pytest.raises(fg.DMCError) as e:
        extractor.compact_mesh(v, q)
    assert e.value.status == 7
    q = torch.tensor([[0, 1, 2, 3]], dtype=torch.int32, device="cuda")
    with pytest.raises(fg.DMCError) as e:
        extractor.compact_mesh(v, q, out_vertices=v)                               # output overlaps input
    assert e.value.status == 1
    out = extractor.compact_mesh(v, q)
    assert out.shape[0] == 4 and q.cpu().tolist() == [[0, 1, 2, 3]]
