"""CPU oracle: cross-check against the pure-Python restatement, hand-derived
single-cell answers, golden fixtures and mesh invariants."""
import glob
import os
from collections import Counter

import numpy as np
import pytest

import oracle
import refpy

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bits_equal(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_pure_python_restatement(seed):
    rng = np.random.default_rng(seed)
    shape = tuple(int(s) for s in rng.integers(2, 7, 3))
    if seed % 3 == 0:
        vol, iso = rng.integers(0, 4, shape).astype(np.uint16), 2.0
    else:
        vol, iso = rng.normal(size=shape).astype(np.float32), float(rng.normal() * 0.3)
    mn = (-1.5, 0.25, 2.0) if seed % 2 else (0, 0, 0)
    mx = (2.5, 3.0, 7.0) if seed % 2 else None
    V, Q = refpy.extract(vol, iso, mn, mx)
    r = oracle.extract(vol, mn, mx, iso)
    ok = ~np.isnan(V).any(1)  # refpy leaves the reference-undefined vertices as NaN
    assert V.shape == r["vertices"].shape
    assert _bits_equal(V[ok], r["vertices"][ok])
    assert np.array_equal(Q, r["quads"])


@pytest.mark.parametrize("config", range(1, 255))
def test_single_cell_every_config(config):
    # One cell, corners -1 (inside) / +1 (outside), iso 0: every crossing is an
    # edge midpoint.  Only the cell's own edges 6, 9, 10 have an owner inside
    # the volume, so a dual vertex averages the midpoints of its patch's
    # edges among 6, 9, 10; a patch with none of them gets the mean of all its
    # midpoints.  No quads: every ring leaves the volume.
    import gen_tables
    lut, nv, _ = gen_tables.build()
    corner = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    vol = np.ones((2, 2, 2), np.float32)
    for i, (x, y, z) in enumerate(corner):
        if (config >> i) & 1:
            vol[z, y, x] = -1.0
    r = oracle.extract(vol, iso=0.0)
    mid = [np.mean([corner[a], corner[b]], axis=0) for a, b in gen_tables.EDGES]
    owned = [e for e in (6, 9, 10) if ((config >> gen_tables.EDGES[e][0]) & 1) != ((config >> gen_tables.EDGES[e][1]) & 1)]
    n_iso = nv[0][config]
    assert len(r["vertices"]) == n_iso + len(owned)
    assert len(r["quads"]) == 0
    for m in range(n_iso):
        edges = [e for e in range(12) if lut[0][config][e] == m]
        use = [e for e in edges if e in (6, 9, 10)] or edges
        np.testing.assert_allclose(r["vertices"][m], np.mean([mid[e] for e in use], axis=0), rtol=0, atol=1e-6)
    for k, e in enumerate(owned):
        np.testing.assert_array_equal(r["vertices"][n_iso + k], mid[e].astype(np.float32))


def test_two_cells_ambiguous_face_uses_lut2():
    # cells (0,0,0) and (1,0,0) share the face x=1.  Config 0x24 (corners 2, 5
    # inside) has its ambiguous face on +x; give the neighbour config 0x09 (its
    # corners 0 and 3... ) chosen so that the shared face alternates and the
    # neighbour is itself one of the 36 ambiguous configs.
    import gen_tables
    _, _, amb = gen_tables.build()
    vol = np.ones((2, 2, 3), np.float32)
    # points: x in 0..2, y in 0..1, z in 0..1; cell0 corners 2=(1,1,0) 5=(1,0,1)
    vol[0, 1, 1] = -1.0
    vol[1, 0, 1] = -1.0
    c0 = 0x24
    # neighbour cell (1,0,0): its corners 0=(1,0,0),3=(1,1,0)=in,4=(1,0,1)=in,7=(1,1,1)
    # config so far: corner3 and corner4 inside -> 0x18, an ambiguous config
    assert amb[c0] != 255 and amb[0x18] != 255
    r = oracle.extract(vol, iso=0.0)
    assert r["n_active"] == 2
    assert r["n_lut2"] == 2


def test_sphere_is_closed_oriented_manifold():
    from framework_gb300 import fields
    vol = fields.sphere_sdf(64, radius=20.0, noise=0.01, seed=1).numpy()
    r = oracle.extract(vol, iso=0.0)
    q = r["quads"]
    assert q.max() < len(r["vertices"])
    und, dire = Counter(), Counter()
    for a, b, c, d in q.tolist():
        for u, v in ((a, b), (b, c), (c, d), (d, a)):
            und[(min(u, v), max(u, v))] += 1
            dire[(u, v)] += 1
    assert set(und.values()) == {2}
    assert max(dire.values()) == 1  # consistent orientation
    assert len(np.unique(q)) - len(und) + len(q) == 2  # Euler characteristic of a sphere


@pytest.mark.parametrize("case", ["blobs", "offset_extent", "u16_noise"])
def test_fp64_oracle_within_stated_bound(case):
    """FP32 replica against FP64: same topology, vertices within 4 ulp of the
    extent's largest coordinate (tests/fp64bound.py states and derives it)."""
    import fp64bound
    from framework_gb300 import fields
    mn = mx = None
    if case == "blobs":
        vol, iso = fields.gaussian_blobs((40, 36, 30), count=5, sigma=(4.0, 8.0), seed=3).numpy(), 0.5
    elif case == "offset_extent":
        vol, iso = fields.gaussian_blobs((48, 40, 33), count=6, sigma=(4.0, 9.0), seed=7).numpy(), 0.4
        mn, mx = (-300.25, 17.5, 1000.0), (-100.0, 80.0, 1090.5)
    else:
        vol, iso = fields.as_u16_numpy(fields.value_noise_u16((70, 64, 50), base_period=16, seed=5)), 32768.0
    a = oracle.extract(vol, mn, mx, iso=iso)
    b = oracle.extract(vol, mn, mx, iso=iso, precision=1)
    assert np.array_equal(a["quads"], b["quads"])
    assert len(a["vertices"]) > 100
    fp64bound.check(a["vertices"], b["vertices"], vol.shape[::-1], mn, mx)


@pytest.mark.parametrize("path", sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                                         if not os.path.basename(p).startswith("ref_")), ids=os.path.basename)
def test_oracle_reproduces_golden(path):
    g = np.load(path)
    r = oracle.extract(g["volume"], g["xyz_min"], g["xyz_max"], float(g["iso"]))
    assert _bits_equal(r["vertices"], g["vertices"])
    assert np.array_equal(r["quads"], g["quads"])
    assert [r["n_active"], r["n_lut2"], r["n_dropped_quads"], r["n_iso_samples"]] == g["counters"].tolist()
    if len(g["quads"]):
        assert g["quads"].max() < len(g["vertices"])


def test_empty_and_degenerate_volumes():
    assert len(oracle.extract(np.zeros((1, 5, 5), np.float32))["vertices"]) == 0
    assert len(oracle.extract(np.ones((4, 4, 4), np.float32), iso=0.5)["vertices"]) == 0
    r = oracle.extract(np.zeros((2, 2, 2), np.float32), iso=0.0)   # all samples == iso: config 0
    assert len(r["vertices"]) == 0 and r["n_iso_samples"] == 8


# ---- smoothing (dmc.cu:1710-1981) ------------------------------------------

def _reference_sphere(n=21):
    """The reference's own usage example (dmc.cu:2248-2306): |p| on a 21^3 grid over [-5, 5]^3."""
    x = np.array([np.float32(i) / np.float32(n - 1) * np.float32(10.0) + np.float32(-5.0) for i in range(n)], np.float32)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    return np.sqrt(xx * xx + y * y + z * z).astype(np.float32)


@pytest.mark.parametrize("num_smooth", [1, 2, 15])
def test_smoothing_oracle_matches_refpy_on_reference_example(num_smooth):
    vol = _reference_sphere()
    V, Q = refpy.extract(vol, 4.1, (-5, -5, -5), (5, 5, 5), num_smooth=num_smooth)
    o = oracle.extract(vol, (-5, -5, -5), (5, 5, 5), 4.1, num_smooth=num_smooth)
    assert np.array_equal(Q, o["quads"])
    assert np.array_equal(np.nan_to_num(V).view(np.uint32), np.nan_to_num(o["vertices"]).view(np.uint32))


@pytest.mark.parametrize("seed", range(3))
def test_smoothing_oracle_matches_refpy_random(seed):
    rng = np.random.default_rng(300 + seed)
    shape = tuple(int(s) for s in rng.integers(4, 9, 3))
    if seed == 2:
        vol, iso = rng.integers(0, 4, shape).astype(np.uint16), 1.5
    else:
        vol, iso = rng.normal(size=shape).astype(np.float32), float(rng.normal() * 0.2)
    V, Q = refpy.extract(vol, iso, (0, 0, 0), None, num_smooth=3)
    o = oracle.extract(vol, iso=iso, num_smooth=3)
    assert np.array_equal(Q, o["quads"])
    ok = ~np.isnan(V).any(1)  # refpy leaves the reference-undefined vertices as NaN
    assert V.shape == o["vertices"].shape and ok.mean() > 0.5
    assert _bits_equal(V[ok], o["vertices"][ok])


def test_smoothing_keeps_topology_and_moves_vertices():
    vol = _reference_sphere()
    a = oracle.extract(vol, (-5, -5, -5), (5, 5, 5), 4.1)
    b = oracle.extract(vol, (-5, -5, -5), (5, 5, 5), 4.1, num_smooth=5)
    assert np.array_equal(a["quads"], b["quads"])
    assert a["vertices"].shape == b["vertices"].shape
    moved = np.any(a["vertices"] != b["vertices"], axis=1)
    assert moved.mean() > 0.5
    # smoothed vertices stay near the surface (radius 4.1, cell size 0.5)
    r = np.linalg.norm(b["vertices"], axis=1)
    assert np.all(np.abs(r - 4.1) < 0.5)


def test_oracle_independent_of_thread_count():
    """The oracle's parallel passes, including the blocked scans that number
    the active cells and place vertices and quads, give the same mesh bit
    for bit on 1, 3 and 8 threads.  The volume spans many 64 Ki-cell scan
    blocks, and its active cells several."""
    from framework_gb300 import fields
    vol = fields.gyroid((150, 120, 90), 0.35, seed=11).numpy()
    ref = None
    try:
        for threads in (1, 3, 8):
            oracle.set_threads(threads)
            r = oracle.extract(vol, iso=0.05)
            got = (r["vertices"].view(np.uint32), r["quads"], r["n_active"], r["n_dropped_quads"])
            if ref is None:
                ref = got
                assert r["n_active"] > 3 * 65536
            else:
                assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2:] == ref[2:]
    finally:
        oracle.set_threads(os.cpu_count() or 1)
