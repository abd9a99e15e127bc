"""Lookup tables: generator freshness, reference parity, structural invariants."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "framework_gb300", "csrc")
sys.path.insert(0, CSRC)
import gen_tables  # noqa: E402

# The reference checkout is read only when DMC_REFERENCE_DIR names it; the
# parity test against its tables is skipped otherwise.
REF_DIR = os.environ.get("DMC_REFERENCE_DIR", "")
REF_DMC = os.path.join(REF_DIR, "DMC_CUDA", "DMC_CUDA", "src", "dmc.cu") if REF_DIR else ""
PINNED_SHA256 = "13d32b2a4949258ce767c4a16cdaf4226031f948d80280dba79d50f242d5e7c7"


def test_generated_file_is_fresh():
    r = subprocess.run([sys.executable, os.path.join(CSRC, "gen_tables.py"), "--check"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert PINNED_SHA256 in r.stdout


def test_oracle_and_library_use_the_pinned_tables():
    import oracle
    assert oracle.tables_sha256() == PINNED_SHA256
    import framework_gb300 as fg
    assert fg.load_library().dmc_tables_sha256().decode() == PINNED_SHA256


def _parse_reference():
    import re
    src = open(REF_DMC).read()

    def grab(name):
        i = src.index(name)
        j = src.index("{", i)
        depth = 0
        for k in range(j, len(src)):
            if src[k] == "{":
                depth += 1
            elif src[k] == "}":
                depth -= 1
                if depth == 0:
                    break
        body = re.sub(r"//[^\n]*", "", src[j:k + 1])
        return np.array([int(n, 0) for n in re.findall(r"0x[0-9a-fA-F]+|\d+", body)])
    return {n: grab(n + "[") for n in ("config_edge_lut1", "config_edge_lut2", "num_vertex_lut1",
                                       "num_vertex_lut2", "config_2B_3B_lut", "config_2B_3B_ambiguous_face")}


@pytest.mark.skipif(not os.path.exists(REF_DMC), reason="DMC_REFERENCE_DIR does not name a reference checkout")
def test_tables_equal_reference_tables():
    ref = _parse_reference()
    lut, nv, amb = gen_tables.build()
    assert np.array_equal(np.array(lut[0]).ravel(), ref["config_edge_lut1"])
    assert np.array_equal(np.array(lut[1]).ravel(), ref["config_edge_lut2"])
    assert np.array_equal(nv[0], ref["num_vertex_lut1"])
    assert np.array_equal(nv[1], ref["num_vertex_lut2"])
    ref_amb = dict(zip(ref["config_2B_3B_lut"].tolist(), ref["config_2B_3B_ambiguous_face"].tolist()))
    assert ref_amb == {c: f for c, f in enumerate(amb) if f != 255}


def test_lut_rows_are_consistent_with_sign_changes():
    lut, nv, amb = gen_tables.build()
    for which in (0, 1):
        for c in range(256):
            row = lut[which][c]
            for e, (a, b) in enumerate(gen_tables.EDGES):
                crossed = ((c >> a) & 1) != ((c >> b) & 1)
                assert (row[e] != 255) == crossed, (which, c, e)
            ms = [m for m in row if m != 255]
            assert nv[which][c] == (max(ms) + 1 if ms else 0)
            assert sorted(set(ms)) == list(range(nv[which][c]))
    assert max(nv[0]) == 4 and max(nv[1]) == 4


def test_lut2_differs_only_on_the_36_ambiguous_configs():
    lut, nv, amb = gen_tables.build()
    diff = [c for c in range(256) if lut[0][c] != lut[1][c]]
    assert len(diff) == 36
    assert diff == [c for c in range(256) if amb[c] != 255]
    # the ambiguous face really alternates, and 2 or 3 corners are inside
    for c in diff:
        loop = gen_tables.FACES[amb[c]]
        assert all(((c >> loop[i]) & 1) != ((c >> loop[(i + 1) % 4]) & 1) for i in range(4))
        assert bin(c).count("1") in (2, 3)


def test_complement_symmetry_of_patch_structure():
    # complementing a config keeps the crossed edges; patch count may differ only on ambiguous faces
    lut, nv, _ = gen_tables.build()
    for c in range(256):
        if not gen_tables.ambiguous_faces(c):
            assert nv[0][c] == nv[0][255 - c]
