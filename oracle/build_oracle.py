#!/usr/bin/env python3
"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

The flags matter: -ffp-contract=off keeps every float multiply and add separate,
as the FP32 replica requires; OpenMP parallelises the per-cell loops only.
-O3 without -march=native: the same source must build, and give the same
results, on the x86_64 build host and on the aarch64 GPU hosts, and with
contraction off the wider vector units would not change a result bit.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
SO = os.path.join(OUT_DIR, "liboracle.so")
SRC = [os.path.join(HERE, "dmc_oracle.c")]
DEPS = SRC + [os.path.join(HERE, "..", "framework_gb300", "csrc", "dmc_tables.inc")]


def build(force=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(SO):
        so_t = os.path.getmtime(SO)
        if all(os.path.getmtime(d) <= so_t for d in DEPS):
            return SO
    tmp = SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unknown-pragmas",
           "-o", tmp] + SRC
    subprocess.check_call(cmd)
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
