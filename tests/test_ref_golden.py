"""Parity against the reference extractor's own outputs.

tests/golden/ref_*.npz hold small volumes together with the vertices and
triangles that the reference's dmc::run_dmc itself produced on a GB300
(DMC_CUDA/DMC_CUDA/src/dmc.cu, built unmodified by oracle/build_ref.py in
three configurations; tests/golden/make_ref_golden.py made the fixtures and
states how the inputs were screened).  The oracle here, and the CUDA library
in the -m gpu test, must give the same triangles (topology, compaction order,
quad connectivity) as every build, and the same vertices:

  * bit for bit against the "debug" build (the reference's shipped
    configuration, -G) and the "nofma" build (-O3 -fmad=false): neither
    contracts a multiply and an add into one FMA, and neither do we;
  * within 2 ulp of the extent's largest coordinate against the "release"
    build (-O3, FMAs allowed: its lerp p0*(1-t) + p1*t and ijk_to_xyz
    i/size*range + min round once instead of twice per multiply-add).  On
    these fixtures that is at most 1.8e-5 voxel, 3.1e-5 in world units.

Every vertex is compared except the dual vertices of patches without an
in-volume owner edge, which the reference leaves uninitialised
(dmc.cu:1584-1592); the oracle flags them ("ownerless"), and none of them is
referenced by a triangle.
"""
import glob
import os

import numpy as np
import pytest

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))
BIT_EXACT = ("debug", "nofma")
RELEASE_ULPS = 2.0


def load(path):
    g = np.load(path)
    return {k: g[k] for k in g.files}


def referenced(tris, n):
    m = np.zeros(n, bool)
    m[np.asarray(tris, np.int64).ravel()] = True
    return m


def compare(vertices, triangles, ownerless, fx, build):
    """Assert one mesh against one reference build of fixture fx; return the
    largest vertex difference in voxels."""
    rv, rt = fx["vertices_" + build], fx["triangles_" + build]
    assert len(vertices) == len(rv), "vertex count differs from the reference (%s)" % build
    assert np.array_equal(np.asarray(triangles, np.uint32), rt.astype(np.uint32)), "triangles differ (%s)" % build
    assert not (referenced(rt, len(rv)) & ownerless).any()
    keep = ~ownerless
    a, b = np.asarray(vertices, np.float32)[keep], rv[keep]
    dims = np.array(fx["volume"].shape[::-1], np.float64)
    spacing = np.abs(fx["xyz_max"].astype(np.float64) - fx["xyz_min"]) / np.maximum(dims - 1, 1)
    d = np.abs(a.astype(np.float64) - b)
    vox = float((d / spacing).max()) if len(a) else 0.0
    if build in BIT_EXACT:
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "vertices not bit-exact (%s): %g voxel" % (build, vox)
    else:
        M = float(max(np.abs(fx["xyz_min"]).max(), np.abs(fx["xyz_max"]).max()))
        tol = RELEASE_ULPS * float(np.spacing(np.float32(M)))
        assert float(d.max()) <= tol, "vertices differ by %g > %g (%s)" % (float(d.max()), tol, build)
    return vox


@pytest.mark.skipif(not CASES, reason="no reference fixtures")
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
def test_oracle_matches_reference(path):
    fx = load(path)
    r = oracle.extract(fx["volume"], tuple(fx["xyz_min"].tolist()), tuple(fx["xyz_max"].tolist()), float(fx["iso"]))
    assert r["n_iso_samples"] == 0          # the fixtures were screened for samples at the isovalue
    for build in ("debug", "release", "nofma"):
        compare(r["vertices"], r["triangles"], r["ownerless"], fx, build)


def test_fixture_set_is_complete():
    names = {os.path.basename(p)[4:-4] for p in CASES}
    assert {"sphere64", "random_ambiguous", "random_offset_extent", "g_checker"} <= names


@pytest.mark.gpu
@pytest.mark.skipif(not CASES, reason="no reference fixtures")
@pytest.mark.parametrize("path", CASES, ids=os.path.basename)
@pytest.mark.parametrize("algo", ["brick", "simple"])
def test_gpu_matches_reference(extractor, path, algo):
    """The CUDA library (both kernel families, host volume in through dmc_run)
    against the reference's own outputs."""
    fx = load(path)
    mn, mx = tuple(fx["xyz_min"].tolist()), tuple(fx["xyz_max"].tolist())
    ownerless = oracle.extract(fx["volume"], mn, mx, float(fx["iso"]))["ownerless"]
    extractor.set_algo(algo)
    try:
        m = extractor.run(fx["volume"], mn, mx, iso=float(fx["iso"]), triangles=True)
    finally:
        extractor.set_algo("auto")
    for build in ("debug", "release", "nofma"):
        compare(m.vertices, m.triangles, ownerless, fx, build)
