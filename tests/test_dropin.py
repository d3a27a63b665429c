"""The drop-in: LBFFS's own driver (ns.cpp) with its OpenCL section replaced by the C ABI.

CPU: the splice recipe produces a driver that compiles and links against liblbffs_cuda.so
(needs the LBFFS checkout).  GPU: the spliced driver, compiled from its bundled headers,
runs the reference's cavityFlow case inputs end to end (input parsing, boundary setup,
initialisation, write.hpp output) and its restart file matches the CPU oracle.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DROPIN = os.path.join(ROOT, "lbffs_gb300", "driver")
sys.path.insert(0, DROPIN)
import make_dropin  # noqa: E402

REF = os.environ.get("LBFFS_REFERENCE", "/root/reference")


def test_dropin_splices_and_compiles(cuda_lib):
    if not os.path.isdir(os.path.join(REF, "D3Q19_opencl")):
        pytest.skip("LBFFS checkout not present")
    for lat in ("D3Q19", "D3Q27"):
        exe = make_dropin.build(REF, lat)
        assert os.path.exists(exe)
        txt = open(os.path.join(DROPIN, "_dropin", lat, "ns.cpp")).read()
        assert "CL/cl2.hpp" not in txt and "lbffs_cuda.h" in txt and "#include \"write.hpp\"" not in txt


def _set(lines, key, val):
    return [f"{key} {val}" if ln.split()[:1] == [key] else ln for ln in lines]


@pytest.mark.gpu
def test_dropin_cavity_runs_on_gpu_and_matches_oracle(cuda_lib, oracle_built, tmp_path):
    out_dir = os.path.join(DROPIN, "_dropin", "D3Q19")
    if not os.path.exists(os.path.join(out_dir, "inc", "input.hpp")):
        pytest.skip("drop-in bundle not generated (needs the LBFFS checkout where it is built)")
    exe = make_dropin.compile_dropin(out_dir)
    n, steps = 32, 200
    lines = open(os.path.join(out_dir, "cavity", "input.txt")).read().splitlines()
    for k, v in (("nx", n), ("ny", n), ("nz", 1), ("endTimeStep", steps), ("outInterval", 100),
                 ("writeBinary", "true"), ("Fwrite", "true"), ("restart", "false")):
        lines = _set(lines, k, v)
    (tmp_path / "input.txt").write_text("\n".join(lines) + "\n")
    (tmp_path / "boundaryConditions.txt").write_text(open(os.path.join(out_dir, "cavity",
                                                                       "boundaryConditions.txt")).read())
    (tmp_path / "out").mkdir()
    r = subprocess.run([exe], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "Speed:" in r.stdout and "GB300 CUDA step" in r.stdout
    raw = open(tmp_path / "out" / "data.dat", "rb").read()
    hdr = np.frombuffer(raw[:16], dtype=np.int32)
    assert list(hdr) == [steps, n, n, 1]
    f_gpu = np.frombuffer(raw[16:], dtype=np.float32)

    # the same case through the host setup mirror and the CPU oracle (ns.cpp:104-131 units)
    from lbffs_gb300 import case as K
    from oracle import ref as R
    kv = {ln.split()[0]: ln.split()[1] for ln in lines if len(ln.split()) >= 2}
    f32 = np.float32
    L = f32(kv["Lx"]) / f32(n - 1)
    c = f32(kv["uMax"]) / f32(kv["U0"])
    nu = f32(f32(kv["nu"].rstrip("f")) / f32(L * c))
    faces = {"nxMin": K.FaceBC(K.BOUNCEBACK, 0, 0), "nxMax": K.FaceBC(K.BOUNCEBACK, 0, 0),
             "nyMin": K.FaceBC(0, K.BOUNCEBACK, 0), "nyMax": K.FaceBC(0, K.FIXEDVELOCITY, 0, f32(1.0) / c, 0, 0),
             "nzMin": K.FaceBC(), "nzMax": K.FaceBC()}
    cs = K.make_case(n, n, 1, 19, faces, nu=float(nu), rho0=float(kv["rho0"]))
    o = R.OracleSolver(cs, sgs="wale", wall="bb", real="f32")
    o.step(steps)
    err = float(np.abs(f_gpu - o.f).max() / np.abs(o.f).max())
    assert err < 1e-5, err
