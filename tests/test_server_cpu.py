"""Host-side logic of the serving loop, without a GPU: the output-arena
allocator (compiled from the library's own header with g++)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_arena_allocator(tmp_path):
    exe = str(tmp_path / "test_arena")
    src = os.path.join(ROOT, "tests", "cpp", "test_arena.cpp")
    inc = os.path.join(ROOT, "framework_gb300", "csrc")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-Wall", "-I", inc, src, "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr


def test_server_symbols_declared():
    import framework_gb300 as fg
    hdr = open(os.path.join(ROOT, "include", "dmc_gb300.h")).read()
    for name in [n for n in fg.ABI_SYMBOLS if n.startswith("dmc_server_")]:
        assert name + "(" in hdr
