#!/usr/bin/env python3
"""Build the reference extractor itself (test infrastructure only).

The reference's DMC path is CUDA (DMC_CUDA/DMC_CUDA/src/dmc.cu with the
headers dmc.hpp, utils.hpp, cuda_includes.h, helper_math.hpp), so it can only
run on the GPU host, and nothing compiled on the x86 build host runs there.
Two steps:

  stage(ref_dir)  on the host that has the reference checkout: copies those
                  five files unchanged into oracle/_ref/src/ and writes
                  forwarding headers for its Windows-style includes
                  (`#include <thrust\\scan.h>`) into oracle/_ref/shim/.
                  oracle/_ref/ is git-ignored: the copies are build inputs
                  that travel to the GPU host with the working tree, never
                  committed sources.
  build(flavor)   on the GPU host: nvcc for sm_103a, with oracle/ref_shim/ (the
                  texture-reference stand-in that CUDA 13 needs) first on the
                  include path, plus oracle/ref_wrap.cu (C entry points), into
                  oracle/_ref/libdmcref_<flavor>.so.

Flavors: "debug" is the reference's shipped Debug configuration (-G, device
code unoptimised; DMC_CUDA/DMC_CUDA/Debug/dmc.cu.cache), "release" nvcc's
defaults at -O3 (multiply-adds may be contracted into FMAs), "nofma" -O3 with
-fmad=false.  The reference source is not edited: its known faults are kept
off the inputs instead (no sample equal to the isovalue, fewer than 4.19 M
active cells; tests/golden/make_ref_golden.py pre-screens for both).
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
SRC_OUT = os.path.join(REF_OUT, "src")
SHIM_OUT = os.path.join(REF_OUT, "shim")
SHIM = os.path.join(HERE, "ref_shim")
WRAP = os.path.join(HERE, "ref_wrap.cu")
FILES = [("src", "dmc.cu"), ("include", "dmc.hpp"), ("include", "utils.hpp"), ("include", "cuda_includes.h"),
         ("include", "helper_math.hpp")]
FLAVORS = {"debug": ["-G"], "release": ["-O3"], "nofma": ["-O3", "-fmad=false"]}


def stage(ref_dir=None):
    ref_dir = ref_dir or os.environ.get("DMC_REFERENCE_DIR", "")
    src_root = os.path.join(ref_dir, "DMC_CUDA", "DMC_CUDA")
    if not ref_dir or not os.path.isdir(src_root):
        raise RuntimeError("set DMC_REFERENCE_DIR to the reference checkout")
    os.makedirs(SRC_OUT, exist_ok=True)
    os.makedirs(SHIM_OUT, exist_ok=True)
    for sub, name in FILES:
        shutil.copyfile(os.path.join(src_root, sub, name), os.path.join(SRC_OUT, name))
    text = open(os.path.join(SRC_OUT, "dmc.cu")).read()
    for inc in sorted(set(re.findall(r"#include\s*<(thrust\\[A-Za-z_]+\.h)>", text))):
        with open(os.path.join(SHIM_OUT, inc), "w") as f:
            f.write("#include <%s>\n" % inc.replace("\\", "/"))
    return SRC_OUT


def staged():
    return all(os.path.exists(os.path.join(SRC_OUT, n)) for _, n in FILES)


def lib_path(flavor):
    return os.path.join(REF_OUT, "libdmcref_%s.so" % flavor)


def build(flavor="debug", force=False):
    if not staged():
        raise RuntimeError("reference sources not staged in %s (run stage() where the reference is)" % SRC_OUT)
    out = lib_path(flavor)
    if not force and os.path.exists(out):
        return out
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    common = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-Xcompiler", "-fPIC",
              "-I", SHIM, "-I", SHIM_OUT, "-I", SRC_OUT] + FLAVORS[flavor]
    objs = []
    for src in (os.path.join(SRC_OUT, "dmc.cu"), WRAP):
        obj = os.path.join(REF_OUT, "%s.%s.o" % (os.path.basename(src), flavor))
        subprocess.check_call(common + ["-c", src, "-o", obj])
        objs.append(obj)
    tmp = out + ".tmp%d" % os.getpid()
    subprocess.check_call([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", tmp] + objs +
                          ["-cudart", "shared"])
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    if "--stage" in sys.argv:
        print(stage())
    for fl in FLAVORS:
        if "--" + fl in sys.argv:
            print(build(fl, force="--force" in sys.argv))
