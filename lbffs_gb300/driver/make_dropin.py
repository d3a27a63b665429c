"""Splice the C-ABI device section into LBFFS's driver and compile it (integration recipe).

Reads ``D3Q19_opencl/ns.cpp`` / ``D3Q27_opencl/ns.cpp`` from an LBFFS checkout, replaces
the OpenCL include block (ns.cpp:18-35) with the C-ABI headers and everything from the
device section's ``try`` (ns.cpp:382) to the end of main() with ``ns_lbffs_block.inc``,
writes the result to ``lbffs_gb300/driver/_dropin/<lattice>/ns.cpp`` and compiles it against
``liblbffs_cuda.so`` with the checkout's own headers on the include path.  The headers the
driver includes and the inputs of two test cases are copied next to it (``inc/``, ``cavity/``,
``cylinderIBM/``) so the same output can be compiled and run where the checkout is absent.
Nothing of the checkout is committed; the output folder is git-ignored.

usage: python lbffs_gb300/driver/make_dropin.py [--lbffs /path/to/LBFFS] [--no-compile]
       (the checkout: --lbffs, else LBFFS_REFERENCE, else reference_dir()'s default)
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)


def reference_dir() -> str:
    """The LBFFS checkout this recipe reads: LBFFS_REFERENCE, else the build machine's checkout."""
    return os.environ.get("LBFFS_REFERENCE", "/root/reference")


def have_reference(lbffs: str = None) -> bool:
    return os.path.isfile(os.path.join(lbffs or reference_dir(), "D3Q19_opencl", "ns.cpp"))


def splice(ns_cpp: str) -> str:
    start = ns_cpp.index("//-- For OpenCL")
    end = ns_cpp.index("#endif", ns_cpp.index("#ifndef DEVICE")) + len("#endif")
    head = ns_cpp[:start] + '#include "lbffs_cuda.h"\n#include "lbffs_cl_compat.hpp"\n#include <cstdlib>\n' + \
        ns_cpp[end:]
    cut = head.index("    try\n    {")
    return head[:cut] + '#include "ns_lbffs_block.inc"\n'


BUNDLE_SRC = ["base.hpp", "input.hpp", "stl.hpp", "walls.hpp", "setBoundaryConditions.hpp"]
BUNDLE_LAT = ["{L}.hpp", "initialization.hpp", "restart.hpp", "write.hpp"]


def bundle(lbffs: str, lattice: str, out_dir: str) -> None:
    """Copy the headers the spliced driver includes, and the cavity case inputs, next to it so the
    build output can be compiled and run on a machine without the checkout."""
    import shutil
    inc = os.path.join(out_dir, "inc")
    os.makedirs(inc, exist_ok=True)
    for f in BUNDLE_SRC:
        shutil.copy(os.path.join(lbffs, "src", f), inc)
    for f in BUNDLE_LAT:
        shutil.copy(os.path.join(lbffs, f"{lattice}_opencl", f.format(L=lattice)), inc)
    for name, src, files in (("cavity", "cavityFlow", ("input.txt", "boundaryConditions.txt")),
                             ("cylinderIBM", "flowAroundCylinderIBM", ("input.txt", "boundaryConditions.txt",
                                                                       "cylinder.stl"))):
        case = os.path.join(out_dir, name)
        os.makedirs(case, exist_ok=True)
        for f in files:
            shutil.copy(os.path.join(lbffs, "testCases", src, f), case)


def compile_dropin(out_dir: str, lbffs: str = None, lattice: str = None) -> str:
    """Compile <out_dir>/ns.cpp; headers from the checkout when given, else from the bundle."""
    out_cpp = os.path.join(out_dir, "ns.cpp")
    exe = os.path.join(out_dir, "ns.cuda")
    incs = [f"-I{os.path.join(lbffs, 'src')}", f"-I{os.path.join(lbffs, lattice + '_opencl')}"] if lbffs else \
        [f"-I{os.path.join(out_dir, 'inc')}"]
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-w", f"-I{os.path.join(ROOT, 'include')}", f"-I{HERE}",
           f"-I{os.path.join(ROOT, 'oracle', 'boost_stub')}", *incs, out_cpp, "-o", exe, f"-L{PKG}", "-llbffs_cuda",
           f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("drop-in compile failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    return exe


def build(lbffs: str, lattice: str, compile_it: bool = True) -> str:
    src_dir = os.path.join(lbffs, f"{lattice}_opencl")
    with open(os.path.join(src_dir, "ns.cpp")) as fh:
        text = splice(fh.read())
    out_dir = os.path.join(HERE, "_dropin", lattice)
    os.makedirs(out_dir, exist_ok=True)
    bundle(lbffs, lattice, out_dir)
    out_cpp = os.path.join(out_dir, "ns.cpp")
    with open(out_cpp, "w") as fh:
        fh.write(text)
    if compile_it:
        return compile_dropin(out_dir, lbffs, lattice)
    return out_cpp


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--lbffs", default=reference_dir())
    ap.add_argument("--no-compile", action="store_true")
    args = ap.parse_args(argv)
    for lat in ("D3Q19", "D3Q27"):
        print(build(args.lbffs, lat, not args.no_compile))
    return 0


if __name__ == "__main__":
    sys.exit(main())
