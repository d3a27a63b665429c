"""Build recipe for ``oracle/_ref``: the reference's own step kernels compiled as C.

Test infrastructure only.  Reads ``D3Q19_opencl/kernel.cl`` and
``D3Q27_opencl/kernel.cl`` from the reference checkout (default
``/root/reference``, override with ``LBFFS_REFERENCE``), applies the oracle
patch set by text substitution, writes the patched sources into
``oracle/_ref/`` and compiles them with ``ref_shim.h`` + ``ref_driver.c`` into
shared libraries there.  Nothing from the reference is written anywhere else.

Patch set (each one is a mechanical substitution with an exact anchor; the
build fails loudly if an anchor is missing):

* P1 ``sgs=smag``: the live SGS call (WALE, D3Q19 kernel.cl:3631 /
  D3Q27 kernel.cl:2816) is replaced by the reference's own commented
  Smagorinsky-with-damping line (D3Q19 kernel.cl:3628 / D3Q27 2814).
  ``sgs=wale`` keeps the as-shipped model.
* P2 ``wall=ibb`` (D3Q19 only): D3Q19's ``internalWallBC`` (kernel.cl:1926,
  simple bounce-back) is replaced by D3Q27's Filippova-Hanel / Mei-Luo-Shyy
  version (D3Q27 kernel.cl:1823-1897) with the loop bound set to 19.
* P3 (always): neighbour reads of rho/u/v/w inside the step see the previous
  step.  The kernel gains ``rhoPrev/uPrev/vPrev/wPrev`` arguments (a snapshot
  the driver takes before each step) which are passed to fixedVelocityBC,
  fixedDensityBC, wallFunctionBC and internalWallBC; WALE's finite
  differences read neighbours from the snapshot and the own cell from the
  freshly updated value (the value the work-item itself just wrote).
* P4 (always): the IBM spread stores the atomic-add result back over the
  sum (D3Q19 kernel.cl:3760-3762); the patched form accumulates with ``+=``
  and the driver runs the spread serially.  ``k_Force`` declares ``solid`` as
  ``float*`` (kernel.cl:3784) while receiving the u8 buffer; it is retyped.
* P5 ``real=f64``: ``-Dfloat=double`` plus REF_DOUBLE in the shim.

The host geometry code (``src/walls.hpp`` / ``src/stl.hpp``) is compiled
by the same recipe into ``voxel_ref19`` / ``voxel_ref27`` with ``boost_stub/`` standing in for
the one Boost call it uses, ``src/setBoundaryConditions.hpp`` into ``case_ref``, and the output
step ``D3Q<Q>_opencl/write.hpp`` into ``output_ref19`` / ``output_ref27``.

Usage: ``python oracle/build_ref.py [--jobs N]``.  Without the reference
checkout (e.g. on a machine the tree was copied to) it compiles the patched
sources already present in ``oracle/_ref`` and exits 0 if there are none.
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF = os.environ.get("LBFFS_REFERENCE", "/root/reference")


def _read(rel):
    with open(os.path.join(REF, rel)) as fh:
        return fh.read()


def _sub_once(text, old, new, what):
    n = text.count(old)
    if n < 1:
        raise SystemExit(f"build_ref: anchor for {what} not found")
    return text.replace(old, new)


def _function(text, signature_start):
    """Return (start, end) of a top-level C function beginning with signature_start."""
    s = text.find(signature_start)
    if s < 0:
        raise SystemExit(f"build_ref: function {signature_start!r} not found")
    e = text.find("\n}\n", s)
    if e < 0:  # last function of the file
        e = text.rfind("\n}")
        return s, len(text) if e < 0 else e + 2
    return s, e + 3


def patch_kernel(q, sgs, wall):
    src = _read(f"D3Q{q}_opencl/kernel.cl")

    # P3: snapshot arguments on the step kernel.
    src = _sub_once(
        src,
        "__kernel void k_streamingCollision // Pull\n(\n",
        "__kernel void k_streamingCollision // Pull\n(\n"
        "   __global float* rhoPrev, __global float* uPrev, __global float* vPrev, __global float* wPrev,\n",
        "kernel signature",
    )
    src = _sub_once(src, "fixedVelocityBC(ft, rhoList, u0", "fixedVelocityBC(ft, rhoPrev, u0", "fixedVelocityBC call")
    src = _sub_once(src, "fixedDensityBC(ft, 1.f, uList, vList, wList,", "fixedDensityBC(ft, 1.f, uPrev, vPrev, wPrev,",
                    "fixedDensityBC call")
    src = _sub_once(src, "wallFunctionBC(ft, rhoList, uList, vList, wList,", "wallFunctionBC(ft, rhoPrev, uPrev, vPrev, wPrev,",
                    "wallFunctionBC call")
    src = _sub_once(src, "upID, omega, tauSGS, rhoList, uList, vList, wList, cx,",
                    "upID, omega, tauSGS, rhoPrev, uPrev, vPrev, wPrev, cx,", "internalWallBC call")

    # P3 for WALE: a copy of waleTauSGS whose neighbour reads see the snapshot.
    s, e = _function(src, "float waleTauSGS(")
    wale = src[s:e]
    wale = wale.replace("float waleTauSGS(", "float waleTauSGS_p3(", 1)
    wale = re.sub(r"const float LES\)",
                  "const float* uPrev, const float* vPrev, const float* wPrev, const float LES)", wale, count=1)
    wale = re.sub(r"([uvw])List\[(index1d\([^\]]*\))\]",
                  r"(((\2) == index1d(i,j,k,nx,ny)) ? \1List[\2] : \1Prev[\2])", wale)
    if "gradU(&dudx" in wale:
        # D3Q27's WALE takes its gradient from gradU (D3Q27 kernel.cl:1993-2025); give it the same view.
        gs, ge = _function(src, "void gradU(")
        grad = src[gs:ge].replace("void gradU(", "void gradU_p3(", 1)
        grad = re.sub(r"float\* wList\)", "float* wList, const float* uPrev, const float* vPrev, const float* wPrev)",
                      grad, count=1)
        grad = re.sub(r"([uvw])List\[(index1d\([^\]]*\))\]",
                      r"(((\2) == index1d(i,j,k,nx,ny)) ? \1List[\2] : \1Prev[\2])", grad)
        wale = wale.replace("gradU(&dudx", "gradU_p3(&dudx").replace(
            "nx, ny, nz, uList, vList, wList);", "nx, ny, nz, uList, vList, wList, uPrev, vPrev, wPrev);")
        wale = grad + "\n" + wale
    src = src[:e] + "\n" + wale + src[e:]
    live = "tauSGSList[ic] = waleTauSGS(i,j,k,nx,ny,nz,uList,vList,wList,LES);"
    if sgs == "smag":
        src = _sub_once(src, live,
                        "tauSGSList[ic] = smagorinskyTauSGS(ft, rho, u, v, w, omega, LES, sdf, cx, cy, cz, wt, REF_CS, 1);",
                        "SGS selection")
    else:
        src = _sub_once(src, live,
                        "tauSGSList[ic] = waleTauSGS_p3(i,j,k,nx,ny,nz,uList,vList,wList,uPrev,vPrev,wPrev,LES);",
                        "SGS selection")

    # P2: D3Q19 interpolated bounce-back from the D3Q27 formula.
    if q == 19 and wall == "ibb":
        q27 = _read("D3Q27_opencl/kernel.cl")
        s27, e27 = _function(q27, "void internalWallBC(")
        ibb = q27[s27:e27].replace("for(int q = 1; q < 27; q++)", "for(int q = 1; q < 19; q++)")
        s19, e19 = _function(src, "void internalWallBC(")
        src = src[:s19] + ibb + src[e19:]

    # P4: IBM spread accumulates; k_Force sees the u8 solid flags.
    src, n = re.subn(r"(G[xyz]IBM)\[icBoxPoint\] = atom_add_float\(&G[xyz]IBM\[icBoxPoint\],([^;]*)\);",
                     r"\1[icBoxPoint] += \2;", src)
    if n != 3:
        raise SystemExit("build_ref: IBM spread anchor not found")
    s, e = _function(src, "__kernel void k_Force")
    body = src[s:e].replace("__global float* solid,", "__global unsigned char* solid,")
    src = src[:s] + body + src[e:]
    return src


def build_one(q, sgs, wall, real, jobs_log):
    name = f"ref_d3q{q}_{sgs}_{wall}_{real}"
    ksrc = os.path.join(OUT, f"kernel_d3q{q}_{sgs}_{wall}.c")
    so = os.path.join(OUT, f"lib{name}.so")
    defs = [f"-DREF_Q={q}", f"-DREF_KERNEL_FILE=\"{ksrc}\""]
    if real == "f64":
        defs += ["-Dfloat=double", "-DREF_DOUBLE=1"]
    cmd = ["gcc", "-std=gnu11", "-O2", "-ffp-contract=off", "-fno-strict-aliasing", "-fno-semantic-interposition", "-fopenmp", "-fPIC", "-shared",
           "-w", f"-I{HERE}", *defs, os.path.join(HERE, "ref_driver.c"), "-o", so, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        jobs_log.append(f"{name}: {r.stderr[-2000:]}")
        return False
    return True


def build_voxel(q, jobs_log):
    exe = os.path.join(OUT, f"voxel_ref{q}")
    lat = os.path.join(REF, f"D3Q{q}_opencl")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fopenmp", "-w", f"-DVOX_Q={q}",
           f"-I{os.path.join(HERE, 'boost_stub')}", f"-I{os.path.join(REF, 'src')}", f"-I{lat}",
           os.path.join(HERE, "voxel_driver.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        jobs_log.append(f"voxel_ref{q}: {r.stderr[-2000:]}")
        return False
    return True


def build_output(q, jobs_log):
    exe = os.path.join(OUT, f"output_ref{q}")
    lat = os.path.join(REF, f"D3Q{q}_opencl")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", f"-DOUT_Q={q}",
           f"-I{os.path.join(HERE, 'boost_stub')}", f"-I{os.path.join(REF, 'src')}", f"-I{lat}",
           os.path.join(HERE, "output_driver.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        jobs_log.append(f"output_ref{q}: {r.stderr[-2000:]}")
        return False
    return True


def build_case(jobs_log):
    exe = os.path.join(OUT, "case_ref")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-w", f"-I{os.path.join(REF, 'src')}",
           os.path.join(HERE, "case_driver.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        jobs_log.append(f"case_ref: {r.stderr[-2000:]}")
        return False
    return True


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    args = ap.parse_args(argv)
    have_ref = os.path.isdir(os.path.join(REF, "D3Q19_opencl"))
    os.makedirs(OUT, exist_ok=True)
    variants = []
    for q in (19, 27):
        walls = ("bb", "ibb") if q == 19 else ("ibb",)
        for sgs in ("smag", "wale"):
            for wall in walls:
                ksrc = os.path.join(OUT, f"kernel_d3q{q}_{sgs}_{wall}.c")
                if have_ref:
                    with open(ksrc, "w") as fh:
                        fh.write(patch_kernel(q, sgs, wall))
                elif not os.path.exists(ksrc):
                    continue
                for real in ("f32", "f64"):
                    so = os.path.join(OUT, f"libref_d3q{q}_{sgs}_{wall}_{real}.so")
                    if have_ref or not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(ksrc):
                        variants.append((q, sgs, wall, real))
    if not have_ref and not variants:
        print("build_ref: reference checkout and generated sources absent (or up to date); nothing to build")
        return 0
    log = []
    with ThreadPoolExecutor(args.jobs) as ex:
        futs = [ex.submit(build_one, *v, log) for v in variants]
        if have_ref:
            futs += [ex.submit(build_voxel, q, log) for q in (19, 27)]
            futs += [ex.submit(build_output, q, log) for q in (19, 27)]
            futs.append(ex.submit(build_case, log))
        ok = all(f.result() for f in futs)
    if not ok:
        print("\n".join(log), file=sys.stderr)
        return 1
    print(f"build_ref: built {len(variants)} kernel libraries into {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
