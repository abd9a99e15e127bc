"""The C++ compatibility header (include/dmc_compat.hpp) and the OBJ writer.

The header is compiled with g++ against the library exactly as a caller of
the reference's dmc::run_dmc would use it.  On the CPU the program must build,
link and report the library's error; on a GPU its mesh must equal the
Python path's and its OBJ file must follow the reference's dump_obj format."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build_compat(tmp_path):
    import framework_gb300 as fg
    from framework_gb300 import build
    build.build()
    exe = str(tmp_path / "compat_main")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA, "include"),
           os.path.join(ROOT, "tests", "cpp", "compat_main.cpp"), "-o", exe,
           "-L", os.path.dirname(build.LIB), "-ldmc_gb300", "-Wl,-rpath," + os.path.dirname(build.LIB)]
    subprocess.check_call(cmd)
    del fg
    return exe


def _sphere(n=21):
    x = np.array([np.float32(i) / np.float32(n - 1) * np.float32(10.0) + np.float32(-5.0) for i in range(n)], np.float32)
    z, y, xx = np.meshgrid(x, x, x, indexing="ij")
    return np.sqrt(xx * xx + y * y + z * z).astype(np.float32)


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_compat_header_builds_and_reports_errors(tmp_path):
    exe = _build_compat(tmp_path)
    out = subprocess.run([exe, "21", "4.1"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    import torch
    if not torch.cuda.is_available():
        assert out.stdout.startswith("error ")


def test_write_obj_format(tmp_path):
    import framework_gb300 as fg
    v = np.array([[0.5, -1.25, 3.0], [1e-7, 123456.789, -0.0], [2, 3, 4]], np.float32)
    t = np.array([[0, 1, 2], [2, 1, 0]], np.uint32)
    p = str(tmp_path / "m.obj")
    fg.write_obj(p, v, t)
    want = "".join("v %g %g %g\n" % tuple(float(c) for c in r) for r in v)
    want += "".join("f %d %d %d\n" % tuple(int(i) + 1 for i in r) for r in t)
    assert open(p).read() == want
    q = np.array([[0, 1, 2, 0]], np.uint32)
    fg.write_obj(p, v, q)
    assert open(p).read().endswith("f 1 2 3 1\n")
    with pytest.raises(fg.DMCError):
        fg.write_obj(p, v, np.array([[0, 1, 3]], np.uint32))   # index out of range


@pytest.mark.gpu
def test_compat_matches_python_path(tmp_path):
    import framework_gb300 as fg
    exe = _build_compat(tmp_path)
    obj = str(tmp_path / "sphere.obj")
    out = subprocess.run([exe, "21", "4.1", obj], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    nv, nt = (int(x) for x in out.stdout.split())
    vol = _sphere(21)
    with fg.Extractor(0) as ex:
        m = ex.run(vol, (-5, -5, -5), (5, 5, 5), 4.1, triangles=True)
    assert (nv, nt) == (len(m.vertices), len(m.triangles))
    lines = open(obj).read().splitlines()
    vs = np.array([[float(c) for c in l.split()[1:]] for l in lines if l.startswith("v ")], np.float32)
    fs = np.array([[int(c) for c in l.split()[1:]] for l in lines if l.startswith("f ")], np.int64)
    assert np.allclose(vs, m.vertices, rtol=1e-5, atol=1e-5)
    assert np.array_equal(fs - 1, m.triangles.astype(np.int64))
