"""GPU parity: the CUDA extractor against the CPU oracle and the golden
fixtures, through the C ABI.  Topology and counts must be identical; vertex
positions must match bit for bit (FP32, same operation order)."""
import glob
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
ALGOS = ["simple", "brick"]


def _bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def _check(mesh, ref):
    assert mesh.vertices.shape == ref["vertices"].shape
    assert mesh.quads.shape == ref["quads"].shape
    assert np.array_equal(mesh.quads, ref["quads"])
    bad = np.flatnonzero((mesh.vertices.view(np.uint32) != ref["vertices"].view(np.uint32)).any(1))
    assert bad.size == 0, "first differing vertices %s: gpu %s oracle %s" % (
        bad[:5], mesh.vertices[bad[:5]], ref["vertices"][bad[:5]])
    tri = oracle.quads_to_triangles(ref["quads"])
    assert np.array_equal(mesh.triangles, tri)


def _supported(ex, algo):
    ex.set_algo(algo)


@pytest.fixture(params=ALGOS)
def algo_extractor(request, extractor):
    extractor.set_algo(request.param)
    yield extractor, request.param
    extractor.set_algo("auto")


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                                         if not os.path.basename(p).startswith("ref_")), ids=os.path.basename)
def test_golden(algo_extractor, path):
    ex, algo = algo_extractor
    g = np.load(path)
    ref = dict(vertices=g["vertices"], quads=g["quads"])
    m = ex.run(g["volume"], g["xyz_min"], g["xyz_max"], float(g["iso"]))
    _check(m, ref)
    st = ex.stats()
    assert [st["n_active_cells"], st["n_lut2_cells"], st["n_dropped_quads"]] == g["counters"][:3].tolist()


def test_sphere_64_c1(algo_extractor):
    from framework_gb300 import fields
    ex, _ = algo_extractor
    vol = fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).numpy()
    _check(ex.run(vol, iso=0.0), oracle.extract(vol, iso=0.0))


@pytest.mark.parametrize("seed", range(6))
def test_random_fields(algo_extractor, seed):
    ex, _ = algo_extractor
    rng = np.random.default_rng(100 + seed)
    shape = tuple(int(s) for s in rng.integers(3, 70, 3))
    if seed % 2:
        vol, iso = rng.integers(0, 5, shape).astype(np.uint16), 2.0
    else:
        vol, iso = rng.normal(size=shape).astype(np.float32), float(rng.normal() * 0.2)
    mn, mx = (-3.0, 0.5, 1.0), (4.0, 2.5, 9.0)
    _check(ex.run(vol, mn, mx, iso), oracle.extract(vol, mn, mx, iso))


@pytest.mark.parametrize("dims", [(2, 2, 2), (3, 2, 2), (2, 40, 3), (70, 2, 5), (33, 65, 2), (129, 31, 3), (257, 9, 4)])
def test_thin_and_ragged_shapes(algo_extractor, dims):
    from framework_gb300 import fields
    ex, _ = algo_extractor
    nx, ny, nz = dims
    vol = fields.gyroid(dims, 0.7, noise=0.05, seed=sum(dims)).numpy()
    assert vol.shape == (nz, ny, nx)
    _check(ex.run(vol, iso=0.05), oracle.extract(vol, iso=0.05))


def test_noise_u16_medium(algo_extractor):
    from framework_gb300 import fields
    ex, _ = algo_extractor
    vol = fields.as_u16_numpy(fields.value_noise_u16((96, 80, 72), base_period=32, seed=7))
    r = oracle.extract(vol, iso=32768.0)
    _check(ex.run(vol, iso=32768.0), r)


@pytest.mark.parametrize("iso", [-3.0, 0.0, 0.5, 1.0, 1.5, 32767.5, 32768.0, 65534.5, 65535.0, 65535.5, 70000.0])
def test_u16_thresholds_wide(algo_extractor, iso):
    """uint16 volumes wide enough (x a multiple of 4, at least 128 columns) for
    the brick path's four-samples-per-load, two-per-word compare, at isovalues
    on and between the extreme sample values (nothing or everything below;
    "at or below" differing from "below")."""
    ex, _ = algo_extractor
    rng = np.random.default_rng(77)
    shape = (23, 37, 256)
    vol = np.array([0, 1, 32768, 65535], np.uint16)[rng.integers(0, 4, shape)]
    some = rng.random(shape) < 0.2                      # and a fifth anywhere in the range
    vol[some] = rng.integers(0, 65536, int(some.sum())).astype(np.uint16)
    _check(ex.run(vol, iso=iso), oracle.extract(vol, iso=iso))


def test_blobs_128(algo_extractor):
    from framework_gb300 import fields
    ex, _ = algo_extractor
    vol = fields.gaussian_blobs((128, 128, 128), count=32, sigma=(8.0, 32.0), seed=2).numpy()
    _check(ex.run(vol, iso=0.5), oracle.extract(vol, iso=0.5))


def test_empty_inputs(extractor):
    for vol in (np.zeros((1, 4, 4), np.float32), np.ones((5, 5, 5), np.float32), np.zeros((3, 3, 3), np.uint16)):
        m = extractor.run(vol, iso=0.5)
        assert len(m.vertices) == 0 and len(m.quads) == 0


def test_device_api_matches_host_api(extractor):
    import torch
    from framework_gb300 import fields
    vol = fields.gaussian_blobs((80, 70, 60), count=8, sigma=(5.0, 12.0), seed=5)
    ref = oracle.extract(vol.numpy(), iso=0.5)
    d = vol.cuda()
    V, Q = len(ref["vertices"]), len(ref["quads"])
    # too small: overflow status carries the needed counts
    with pytest.raises(Exception) as ei:
        extractor.extract_device(d, iso=0.5, vertices=torch.empty((1, 3), device="cuda"), quads=torch.empty((1, 4), dtype=torch.int32, device="cuda"))
    assert getattr(ei.value, "counts", None) == (V, Q)
    vb = torch.empty((V, 3), device="cuda")
    qb = torch.empty((Q, 4), dtype=torch.int32, device="cuda")
    tb = torch.empty((2 * Q, 3), dtype=torch.int32, device="cuda")
    nv, nq = extractor.extract_device(d, iso=0.5, vertices=vb, quads=qb, triangles=tb)
    assert (nv, nq) == (V, Q)
    assert _bits_equal(vb.cpu().numpy(), ref["vertices"])
    assert np.array_equal(qb.cpu().numpy().view(np.uint32), ref["quads"])
    assert np.array_equal(tb.cpu().numpy().view(np.uint32), ref["triangles"])


def test_reference_shaped_module_api():
    import framework_gb300 as fg
    from framework_gb300 import fields
    vol = fields.sphere_sdf(21, radius=4.1 * 2, noise=0.0).numpy()
    fg.setup_device_luts()
    v, t = fg.run_dmc(vol, (-5, -5, -5), (5, 5, 5), 0.0)
    fg.cleanup_device_luts()
    r = oracle.extract(vol, (-5, -5, -5), (5, 5, 5), 0.0)
    assert _bits_equal(v, r["vertices"]) and np.array_equal(t, r["triangles"])


def _streamed_case(kind):
    from framework_gb300 import fields
    if kind == "u16":
        vol = fields.value_noise_u16((150, 70, 261), base_period=16, seed=12)
        return fields.as_u16_numpy(vol), 32768.0
    return fields.gaussian_blobs((140, 90, 300), seed=5).numpy(), 0.5


def _host_out(V, Q, pinned):
    import torch
    if pinned:
        return (torch.empty((V, 3), dtype=torch.float32, pin_memory=True).numpy(),
                torch.empty((Q, 4), dtype=torch.int32, pin_memory=True).numpy(),
                torch.empty((2 * Q, 3), dtype=torch.int32, pin_memory=True).numpy())
    return np.empty((V, 3), np.float32), np.empty((Q, 4), np.int32), np.empty((2 * Q, 3), np.int32)


@pytest.mark.parametrize("kind", ["u16", "f32"])
def test_run_into_streamed(kind):
    """dmc_run_into in z slabs (upload, extraction and download overlapped)
    returns the unstreamed mesh bit for bit for several slab counts, with and
    without triangles, into pinned and pageable buffers.  A fresh context
    (no device output buffers yet), device buffers grown for a smaller mesh,
    and host buffers that are too small all behave as unstreamed."""
    import framework_gb300 as fg
    host, iso = _streamed_case(kind)
    mn, mx = (-1.0, 0.5, 2.0), (3.0, 4.0, 11.0)
    with fg.Extractor(0) as ex:
        ex.set_option(fg.OPT_STREAM_SLABS, 1)
        m = ex.run(host, mn, mx, iso, triangles=True)
        V, Q = len(m.vertices), len(m.quads)
        assert V > 10000 and Q > 5000
        ref = (m.vertices.view(np.uint32), m.quads, m.triangles)

    def check(ex, bufs, tris=True, quads=True):
        hv, hq, ht = bufs
        hv.fill(-1), hq.fill(-1), ht.fill(-1)
        assert ex.run_into(host, hv, hq if quads else None, ht if tris else None, mn, mx, iso) == (V, Q)
        assert np.array_equal(hv.view(np.uint32), ref[0])
        if quads:
            assert np.array_equal(hq.view(np.uint32), ref[1])
        else:
            assert (hq.view(np.uint32) == 0xFFFFFFFF).all()   # not written
        if tris:
            assert np.array_equal(ht.view(np.uint32), ref[2])

    with fg.Extractor(0) as ex:
        # device buffers grown for a small mesh first: the streamed call finds them short
        small = host[:20, :30, :40].copy()
        ms = ex.run(small, None, None, iso)
        sv, sq = len(ms.vertices), len(ms.quads)
        ex.run_into(small, np.empty((sv, 3), np.float32), np.empty((sq, 4), np.int32), None, None, None, iso)
        for slabs in (4, 2, 3, 7, 16, 32):
            ex.set_option(fg.OPT_STREAM_SLABS, slabs)
            for pinned in (True, False):
                bufs = _host_out(V, Q, pinned)
                check(ex, bufs)
                check(ex, bufs, tris=False)
                check(ex, bufs, quads=False)   # the reference's outputs: vertices and triangles
            st = ex.stats()
            assert (st["n_vertices"], st["n_quads"]) == (V, Q)
        hv, hq, ht = _host_out(V, Q, True)
        with pytest.raises(fg.DMCError) as e:
            ex.run_into(host, hv[:V - 1], hq, ht, mn, mx, iso)
        assert e.value.status == 3 and e.value.counts == (V, Q)
        with pytest.raises(fg.DMCError) as e:
            ex.run_into(host, hv, hq[:Q - 1], None, mn, mx, iso)
        assert e.value.status == 3 and e.value.counts == (V, Q)
        check(ex, (hv, hq, ht))       # usable afterwards


def test_run_into_matches_run(extractor):
    """dmc_run_into (caller host buffers, here page-locked) gives dmc_run's mesh."""
    import torch
    import framework_gb300 as fg
    from framework_gb300 import fields
    vol = fields.value_noise_u16((120, 90, 70), base_period=16, seed=9)
    host = fields.as_u16_numpy(vol)
    m = extractor.run(host, (-1, 0, 2), (5, 4, 9), 32768.0, triangles=True)
    V, Q = len(m.vertices), len(m.quads)
    hv = torch.empty((V, 3), dtype=torch.float32, pin_memory=True).numpy()
    hq = torch.empty((Q, 4), dtype=torch.int32, pin_memory=True).numpy()
    ht = torch.empty((2 * Q, 3), dtype=torch.int32, pin_memory=True).numpy()
    for rep in range(2):
        hv.fill(-1), hq.fill(-1), ht.fill(-1)
        nv, nq = extractor.run_into(host, hv, hq, ht, (-1, 0, 2), (5, 4, 9), 32768.0)
        assert (nv, nq) == (V, Q)
        assert np.array_equal(hv.view(np.uint32), m.vertices.view(np.uint32))
        assert np.array_equal(hq.view(np.uint32), m.quads) and np.array_equal(ht.view(np.uint32), m.triangles)
    # pageable numpy buffers and no triangles work the same
    pv, pq = np.empty((V, 3), np.float32), np.empty((Q, 4), np.uint32)
    assert extractor.run_into(host, pv, pq, None, (-1, 0, 2), (5, 4, 9), 32768.0) == (V, Q)
    assert np.array_equal(pv.view(np.uint32), m.vertices.view(np.uint32)) and np.array_equal(pq, m.quads)
    with pytest.raises(fg.DMCError) as e:
        extractor.run_into(host, pv[:V - 1], pq, None, (-1, 0, 2), (5, 4, 9), 32768.0)
    assert e.value.status == 3 and e.value.counts == (V, Q)
    # vertices and triangles only, as dmc::run_dmc returns them
    pt = np.full((2 * Q, 3), 0xFFFFFFFF, np.uint32)
    assert extractor.run_into(host, pv, None, pt, (-1, 0, 2), (5, 4, 9), 32768.0) == (V, Q)
    assert np.array_equal(pt, m.triangles)
    with pytest.raises(fg.DMCError) as e:
        extractor.run_into(host, pv, None, pt[:2 * Q - 2], (-1, 0, 2), (5, 4, 9), 32768.0)
    assert e.value.status == 3 and e.value.counts == (V, Q)
    with pytest.raises(fg.DMCError):
        extractor.run_into(host, pv, None, None, (-1, 0, 2), (5, 4, 9), 32768.0)


def test_run_arrays_own_the_mesh(extractor):
    """dmc_run's arrays wrap the library's buffers without a copy; each one
    stays valid on its own after the Mesh and the other arrays are gone."""
    import gc
    from framework_gb300 import fields
    vol = fields.value_noise_u16((96, 80, 72), base_period=12, seed=4)
    host = fields.as_u16_numpy(vol)
    r = oracle.extract(host, iso=30000.0)
    m = extractor.run(host, iso=30000.0, triangles=True)
    tris = m.triangles[1:]
    verts = m.vertices
    del m
    gc.collect()
    big = [np.ones(1 << 20, np.float64) for _ in range(8)]   # reuse freed memory, if any was freed
    assert np.array_equal(verts.view(np.uint32), r["vertices"].view(np.uint32))
    assert np.array_equal(tris, r["triangles"][1:]) and not verts.flags["OWNDATA"]
    del big
