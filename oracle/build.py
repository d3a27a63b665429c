"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``lbm_oracle.c`` twice -- REAL=float and REAL=double -- into
``oracle/liboracle_f32.so`` / ``oracle/liboracle_f64.so`` with plain gcc
(no FMA contraction, so the FP32 build rounds like the reference's C build).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def build_oracle(verbose=False):
    src = os.path.join(HERE, "lbm_oracle.c")
    deps = [src, os.path.join(HERE, "lbm_oracle_d3q27.h"), os.path.join(HERE, "lbm_oracle_ibm.h")]
    procs = []
    for real, tag in (("float", "f32"), ("double", "f64")):
        out = os.path.join(HERE, f"liboracle_{tag}.so")
        if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
            continue
        cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
               "-Wno-unused-function", f"-DREAL={real}", src, "-o", out, "-lm"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + out)
        if verbose and out:
            print(out)


if __name__ == "__main__":
    build_oracle(verbose=True)
    sys.exit(0)
