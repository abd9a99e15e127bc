"""The CPU oracle under AddressSanitizer (with leak checks) and
UndefinedBehaviorSanitizer: oracle/sanitize_check.c runs every cell
configuration, samples equal to the isovalue, ragged and degenerate shapes,
reversed extents, FP64 mode and smoothing, and checks each mesh's quad
indices.  compute-sanitizer is not available for the device code, so the
host side is where sanitizers run."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_under_sanitizers(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "sanitize_check")
    cmd = [gcc, "-std=c11", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fno-omit-frame-pointer", "-ffp-contract=off", "-Wall", "-Wno-unknown-pragmas",
           "-o", exe, os.path.join(ROOT, "oracle", "sanitize_check.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    if r.returncode != 0 and ("asan" in r.stderr or "ubsan" in r.stderr):
        pytest.skip("no sanitizer runtime for gcc: " + r.stderr.strip().splitlines()[-1])
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "sanitize check: ok" in out.stdout
