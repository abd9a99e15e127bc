"""GPU parity where a few samples equal the isovalue exactly.

The reference's bipolar test (dmc.cu:1101-1106, 1199-1216) separates "below"
from "at": an edge between a sample below the isovalue and one equal to it
is bipolar, one between two equal samples is not.  The brick count sweep
keeps only "below" masks and reads the corners of an active cell one by one
where a sample can be equal.  These cases plant isolated equal samples next
to the places where a brick's bookkeeping could go wrong: the first and
last columns of a 128-column tile, the halo column (the next tile's column
0), the edges of a lane's four columns (3/4), the brick's row 32 (the next
brick's row 0), the first and last planes, on the 4-sample load path
(x extent a multiple of 4, tiles wholly inside) and on the per-column path
(ragged last tile).  Everything is compared bit for bit with the oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

XS = (0, 1, 3, 4, 5, 126, 127, 128, 129, 131, 132, 254, 255, 256, 257)
YS = (0, 1, 30, 31, 32, 33, 63, 64, 65)


def _plant(vol, iso, rng, n_extra=40):
    nz, ny, nx = vol.shape
    zs = sorted({0, 1, nz // 2, nz - 2, nz - 1})
    pts = [(x, y, z) for x in XS for y in YS for z in zs if x < nx and y < ny and (x + y + z) % 3 == 0]
    for _ in range(n_extra):
        pts.append((int(rng.integers(nx)), int(rng.integers(ny)), int(rng.integers(nz))))
    for x, y, z in pts:
        vol[z, y, x] = iso
    return len(pts)


def _check(m, ref):
    assert m.vertices.shape == ref["vertices"].shape and m.quads.shape == ref["quads"].shape
    assert np.array_equal(m.quads, ref["quads"])
    assert np.array_equal(m.vertices.view(np.uint32), ref["vertices"].view(np.uint32))


@pytest.mark.parametrize("nx", [384, 300, 262])
@pytest.mark.parametrize("algo", ["brick", "simple"])
def test_u16_isolated_equal_samples(extractor, algo, nx):
    rng = np.random.default_rng(nx)
    iso = 30000
    vol = rng.integers(20000, 40000, (9, 70, nx)).astype(np.uint16)
    vol[vol == iso] = iso + 1
    n = _plant(vol, iso, rng)
    assert int((vol == iso).sum()) <= n
    extractor.set_algo(algo)
    try:
        m = extractor.run(vol, iso=float(iso))
    finally:
        extractor.set_algo("auto")
    ref = oracle.extract(vol, iso=float(iso))
    _check(m, ref)
    st = extractor.stats()
    assert st["n_active_cells"] == ref["n_active"]


@pytest.mark.parametrize("nx", [384, 262])
def test_f32_isolated_equal_samples(extractor, nx):
    from framework_gb300 import fields
    rng = np.random.default_rng(7 + nx)
    vol = fields.gaussian_blobs((nx, 66, 7), count=12, sigma=(3.0, 9.0), seed=5).numpy()
    iso = np.float32(0.5)
    vol[vol == iso] = np.nextafter(iso, np.float32(1))
    # equal samples only matter next to the surface: plant them where the
    # field is near the isovalue as well as at the fixed places
    near = np.argwhere(np.abs(vol - iso) < 0.05)
    for z, y, x in near[rng.choice(len(near), size=min(60, len(near)), replace=False)]:
        vol[z, y, x] = iso
    _plant(vol, iso, rng, n_extra=0)
    extractor.set_algo("brick")
    try:
        m = extractor.run(vol, iso=float(iso))
    finally:
        extractor.set_algo("auto")
    _check(m, oracle.extract(vol, iso=float(iso)))
