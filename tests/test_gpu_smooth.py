"""Vertex smoothing (num_smooth > 0, dmc.cu:1710-1981) on the GPU against the
CPU oracle: identical topology and bit-identical vertices (both sides use the
same single-precision arithmetic with explicit rounding)."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _reference_sphere(n=21):
    x = np.array([np.float32(i) / np.float32(n - 1) * np.float32(10.0) + np.float32(-5.0) for i in range(n)], np.float32)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    return np.sqrt(xx * xx + y * y + z * z).astype(np.float32)


def _same(m, ref):
    assert np.array_equal(m.quads, ref["quads"])
    assert m.vertices.shape == ref["vertices"].shape
    bad = np.flatnonzero((m.vertices.view(np.uint32) != ref["vertices"].view(np.uint32)).any(1))
    assert bad.size == 0, "first differing vertices %s: gpu %s oracle %s" % (
        bad[:4], m.vertices[bad[:4]], ref["vertices"][bad[:4]])


@pytest.mark.parametrize("num_smooth", [1, 3, 15])
def test_reference_example(extractor, num_smooth):
    """The reference's usage example: 21^3 sphere over [-5,5]^3, iso 4.1, num_smooth 15."""
    vol = _reference_sphere()
    m = extractor.run(vol, (-5, -5, -5), (5, 5, 5), 4.1, num_smooth=num_smooth)
    _same(m, oracle.extract(vol, (-5, -5, -5), (5, 5, 5), 4.1, num_smooth=num_smooth))
    assert m.stats["algo"] == 1          # smoothing runs on the simple path


@pytest.mark.parametrize("seed", range(4))
def test_random_fields(extractor, seed):
    rng = np.random.default_rng(500 + seed)
    shape = tuple(int(s) for s in rng.integers(5, 60, 3))
    if seed % 2:
        vol, iso = rng.integers(0, 6, shape).astype(np.uint16), 2.5
    else:
        from framework_gb300 import fields
        vol = fields.gyroid(shape[::-1], 0.3, seed=seed).numpy()
        iso = float(rng.normal() * 0.2)
    mn, mx = (-2.0, 0.5, 1.0), (3.0, 4.5, 9.0)
    m = extractor.run(vol, mn, mx, iso, num_smooth=4)
    _same(m, oracle.extract(vol, mn, mx, iso, num_smooth=4))


def test_device_form_and_errors(extractor):
    import torch
    import framework_gb300 as fg
    from framework_gb300 import fields
    vol = fields.sphere_sdf(48, radius=15.0, noise=0.01, seed=4).cuda()
    nv, nq = extractor.extract_device(vol, iso=0.0)
    v = torch.empty((nv, 3), device="cuda")
    q = torch.empty((nq, 4), dtype=torch.int32, device="cuda")
    extractor.extract_device(vol, iso=0.0, vertices=v, quads=q, num_smooth=2)
    ref = oracle.extract(vol.cpu().numpy(), iso=0.0, num_smooth=2)
    assert np.array_equal(v.cpu().numpy().view(np.uint32), ref["vertices"].view(np.uint32))
    with pytest.raises(fg.DMCError) as e:        # vertices without the quad ring buffer
        extractor.extract_device(vol, iso=0.0, vertices=v, num_smooth=2)
    assert e.value.status == 1
    extractor.set_algo("brick")
    try:
        with pytest.raises(fg.DMCError) as e:    # the brick path keeps no per-cell offsets
            extractor.extract_device(vol, iso=0.0, vertices=v, quads=q, num_smooth=2)
        assert e.value.status == 6
    finally:
        extractor.set_algo("auto")
