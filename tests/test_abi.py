"""The C ABI library builds, loads without a GPU and exports every entry point
declared in include/*.h (no compute calls here)."""
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+char\s*\*|dmc_status|void|int|uint64_t)\s*\**\s*(dmc_\w+)\s*\(", src, re.M)
    return sorted(set(names))


def test_header_declares_the_reference_replacements():
    d = _declared()
    for name in ("dmc_create", "dmc_destroy", "dmc_run", "dmc_extract_device"):
        assert name in d


def test_library_exports_every_declared_symbol():
    import framework_gb300 as fg
    L = fg.load_library()
    out = subprocess.run(["nm", "-D", "--defined-only", fg.library_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\sT\s(dmc_\w+)", out))
    missing = [n for n in _declared() if n not in exported]
    assert not missing, missing
    for n in _declared():
        assert hasattr(L, n)
    assert fg.ABI_SYMBOLS == [n for n in fg.ABI_SYMBOLS if n in exported]


def test_build_targets_sm_103a_only():
    from framework_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_status_strings_and_version():
    import framework_gb300 as fg
    L = fg.load_library()
    assert b"sm_103a" in L.dmc_version()
    for s in range(8):
        assert L.dmc_status_string(s)


def test_create_without_gpu_fails_cleanly():
    import ctypes
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import framework_gb300 as fg
    L = fg.load_library()
    h = ctypes.c_void_p()
    assert L.dmc_create(ctypes.byref(h), 0) == 1  # DMC_ERR_INVALID_ARG: no such device
    # the CUDA error behind it, as the reference would print it before exiting
    assert L.dmc_last_cuda_error().startswith(b"cudaError")
    assert fg.last_cuda_error().startswith("cudaError")
    with pytest.raises(fg.DMCError):
        fg.Extractor(0)


def test_python_constants_match_the_header():
    """The Python binding's status, dtype, algorithm and option numbers are
    the header's enum values."""
    import re
    import framework_gb300 as fg
    text = open(os.path.join(ROOT, "include", "dmc_gb300.h")).read()
    enum = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(DMC_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    assert {v: k for k, v in fg.STATUS.items()} == {k: v for k, v in enum.items()
                                                    if k == "DMC_OK" or k.startswith("DMC_ERR_")}
    assert fg.DTYPE == {"float32": enum["DMC_F32"], "uint16": enum["DMC_U16"]}
    assert fg.ALGO == {"auto": enum["DMC_ALGO_AUTO"], "simple": enum["DMC_ALGO_SIMPLE"], "brick": enum["DMC_ALGO_BRICK"]}
    for name in ("BRICK_PLANES", "STREAM_SLABS", "FAIL_ALLOCS"):
        assert getattr(fg, "OPT_" + name) == enum["DMC_OPT_" + name]
    cells = re.search(r"#define\s+DMC_NOALLOC_MAX_CELLS\s+(\d+)u?", text)
    assert cells and fg.NOALLOC_MAX_CELLS == int(cells.group(1))
