"""Randomised parity of the brick path against the oracle.

Forty seeded volumes whose shapes straddle the brick geometry: x extents
around multiples of the 128-column tile (and odd ones, which take the
per-column load path), y extents around multiples of the 32-row brick,
z extents of a few planes to a few bricks.  The values are coarsely
quantised, so many samples equal the isovalue (the reference's bipolar
test, dmc.cu:1101-1106, and the count sweep's corner reads for it), and
half the cases use uint16 samples with an integer isovalue.  Every mesh
must equal the oracle's bit for bit, with the same active, LUT2 and
dropped-quad counters."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

XS = (3, 64, 127, 128, 129, 130, 255, 256, 257, 300, 385)
YS = (2, 31, 32, 33, 34, 63, 64, 65, 97)
ZS = (2, 3, 5, 9, 17)


def _case(seed):
    rng = np.random.default_rng(1000 + seed)
    nx, ny, nz = int(rng.choice(XS)), int(rng.choice(YS)), int(rng.choice(ZS))
    if seed % 2:
        levels = int(rng.integers(3, 9))
        vol = rng.integers(0, levels, (nz, ny, nx)).astype(np.uint16) * np.uint16(1000)
        iso = float(1000 * int(rng.integers(1, levels)))
    else:
        vol = (np.round(rng.normal(size=(nz, ny, nx)) * 4) / 4).astype(np.float32)
        iso = float(rng.choice([-0.25, 0.0, 0.25, 0.5]))
    mn = tuple(float(v) for v in rng.uniform(-5, 5, 3))
    mx = tuple(m + float(d) for m, d in zip(mn, rng.uniform(1, 50, 3)))
    return vol, iso, mn, mx


@pytest.mark.parametrize("seed", range(40))
def test_brick_matches_oracle_on_random_shapes(extractor, seed):
    vol, iso, mn, mx = _case(seed)
    extractor.set_algo("brick")
    try:
        m = extractor.run(vol, mn, mx, iso)
        st = extractor.stats()
    finally:
        extractor.set_algo("auto")
    ref = oracle.extract(vol, mn, mx, iso)
    assert m.vertices.shape == ref["vertices"].shape and m.quads.shape == ref["quads"].shape
    assert np.array_equal(m.quads, ref["quads"])
    assert np.array_equal(m.vertices.view(np.uint32), ref["vertices"].view(np.uint32))
    assert st["n_active_cells"] == ref["n_active"]
    assert [st["n_lut2_cells"], st["n_dropped_quads"]] == [ref["n_lut2"], ref["n_dropped_quads"]]
