"""Build recipe for ``lbffs_gb300/liblbffs_cuda.so`` (the C-ABI CUDA library).

Compiles every ``csrc/*.cu`` / ``*.cpp`` translation unit for sm_103a in parallel with nvcc
and links them into one shared library next to this file.  Rebuilds only what changed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblbffs_cuda.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "-I", CSRC, "-I", INCLUDE]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
           [os.path.join(INCLUDE, "lbffs_cuda.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra_flags=None, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    hdrs = _headers()
    units = []  # (source, object, defines)
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")) and f not in ("step_inst.cu", "batch_inst.cu", "bulk_tma.cu"):
            units.append((f, os.path.splitext(f)[0] + ".o", []))
    # batched kernels of the server: one object per storage format
    for st in (0, 1, 2):
        units.append(("batch_inst.cu", f"batch_s{st}.o", [f"-DLBFFS_S={st}"]))
        units.append(("bulk_tma.cu", f"bulk_tma_s{st}.o", [f"-DLBFFS_S={st}"]))
    # the step kernels: one object per (lattice, storage, collision, kernel variant) so they compile
    # in parallel (step_inst.cu lists the parts)
    for q, colls in ((19, (0,)), (27, (0, 1))):
        for st in (0, 1, 2):
            for coll in colls:
                for part in (0, 1, 2, 3):
                    units.append(("step_inst.cu", f"step_q{q}_s{st}_c{coll}_p{part}.o",
                                  [f"-DLBFFS_Q={q}", f"-DLBFFS_S={st}", f"-DLBFFS_C={coll}", f"-DLBFFS_PART={part}"]))
    cmds = []
    objs = []
    for s, o, defs in units:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, o)
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            cmds.append([nvcc(), *ARCH, *NVCC_FLAGS, *defs, *(extra_flags or []), "-c", src, "-o", obj])
    # longest compiles first
    cmds.sort(key=lambda c: ("_c1_" not in c[-1], "step_q27" not in c[-1]))

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(jobs or os.cpu_count() or 4) as ex:
        for cmd, r in ex.map(run, cmds):
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if cmds or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    verbose = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else None
    print(build(verbose=verbose or bool(extra), extra_flags=extra))
