"""Build the CUDA extension library ``libdmc_gb300.so`` in-tree.

Every translation unit is compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``), in parallel, then linked into one shared
library that exports the C ABI declared in include/dmc_gb300.h.  The result
lands in framework_gb300/_build/ (git-ignored) and is rebuilt when a source
or header is newer than it.
"""
import concurrent.futures
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libdmc_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills",
              "--expt-relaxed-constexpr"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build framework_gb300")


def sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")))


def deps():
    d = sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
    d += glob.glob(os.path.join(CSRC, "*.inc")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    return d


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in deps())


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ["-I", os.path.join(ROOT, "include"), "-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and up_to_date():
        return LIB
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if verbose:
        for obj, log in results:
            if log.strip():
                print(log)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + [o for o, _ in results] + ["-lcudart", "-lpthread", "-ldl"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
