"""Record golden vectors of the reference's output step (run here, on the CPU).

oracle/_ref/output_ref19 / output_ref27 run D3Q19_opencl/write.hpp and D3Q27_opencl/write.hpp
(compiled from the reference sources by oracle/build_ref.py) on seeded synthetic arrays.  Every
case is two outputs in a row: the first with zero time means, the second with the means the first
left and new populations, so the fixtures hold the time-mean accumulation too.  Saved per case
and output k (1, 2): the input arrays, the VTK file, data.dat, the host rho / u / v / w / means
after write.hpp, rho_av and timeMean, and write.hpp's console lines for uAve, rho and the force
coefficients.

usage: python tests/golden/make_golden_output.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.path.join(ROOT, "oracle", "_ref")

from lbffs_gb300 import case as K  # noqa: E402

# name: (q, nx, ny, nz, nt, dpdx, c, L, uMax, Dref, forceCoeffs, writeBinary, outInterval)
CASES = {
    "q19_ascii": (19, 10, 8, 6, 1200, 1.0e-5, 2.0, 0.01, 0.5, 4.0, 1, 0, 100),
    "q19_binary": (19, 9, 7, 5, 800, 0.0, 1.5, 0.02, 0.3, 3.0, 0, 1, 50),
    "q27_ascii": (27, 8, 6, 5, 400, 2.0e-6, 1.0, 0.05, 0.2, 2.0, 1, 0, 25),
}


def inputs(q, nx, ny, nz, seed):
    """Seeded arrays of one output: near-equilibrium populations and arbitrary other fields."""
    rng = np.random.default_rng(seed)
    E = nx * ny * nz
    wq = K.lattice(q)[1].astype(np.float64)
    f = (wq[:, None] * (1.0 + 0.02 * (rng.random((q, E)) - 0.5))).astype(np.float32)
    solid = (rng.random(E) < 0.1).astype(np.uint8)
    b1 = np.zeros(E, np.int32)
    b2 = np.zeros(E, np.int32)
    b3 = np.zeros(E, np.int32)
    B1, B2, B3 = (x.reshape(nz, ny, nx) for x in (b1, b2, b3))
    B1[:, :, 0], B1[:, :, -1] = 5, 3
    B2[:, 0, :], B2[:, -1, :] = 1, 4
    B3[0, :, :], B3[-1, :, :] = 0, 1
    sdf = np.where(rng.random(E) < 0.3, np.float32(10000.0), (10.0 * rng.random(E)).astype(np.float32))
    return {
        "f": f.reshape(-1),
        "tauSGS": (0.02 * rng.random(E)).astype(np.float32),
        "omega": (1.5 + 0.4 * rng.random(E)).astype(np.float32),
        "Fwx": (1e-3 * (rng.random(E) - 0.5)).astype(np.float32),
        "Fwy": (1e-3 * (rng.random(E) - 0.5)).astype(np.float32),
        "Fwz": (1e-3 * (rng.random(E) - 0.5)).astype(np.float32),
        "GxIBM": (1e-4 * (rng.random(E) - 0.5)).astype(np.float32),
        "GyIBM": (1e-4 * (rng.random(E) - 0.5)).astype(np.float32),
        "GzIBM": (1e-4 * (rng.random(E) - 0.5)).astype(np.float32),
        "boundary1": b1, "boundary2": b2, "boundary3": b3,
        "sdf": sdf.astype(np.float32),
        "solid": solid,
        "neiSolid": (rng.random(E) < 0.2).astype(np.uint8),
    }


EXT = {np.dtype(np.float32): "f32", np.dtype(np.int32): "i32", np.dtype(np.uint8): "u8"}


def run_case(name, spec, out):
    q, nx, ny, nz, nt, dpdx, c, L, umax, dref, fc, binary, interval = spec
    E = nx * ny * nz
    means = {k: np.zeros(E, np.float32) for k in ("uMean", "vMean", "wMean")}
    time_mean = 0.0
    for k in (1, 2):
        arrs = inputs(q, nx, ny, nz, seed=1000 * k + 10 * len(name) + q)
        if not fc:  # without forceCoeffs the driver never downloads them: its host copies stay zero
            for key in ("Fwx", "Fwy", "Fwz", "GxIBM", "GyIBM", "GzIBM"):
                arrs[key] = np.zeros_like(arrs[key])
        with tempfile.TemporaryDirectory() as td:
            ind = os.path.join(td, "in")
            work = os.path.join(td, "work")
            os.makedirs(ind)
            os.makedirs(os.path.join(work, "out"))
            for key, a in list(arrs.items()) + list(means.items()):
                a.tofile(os.path.join(ind, f"{key}.{EXT[a.dtype]}"))
            step = nt * k
            r = subprocess.run([os.path.join(REF, f"output_ref{q}"), ind, work, str(nx), str(ny), str(nz), str(step),
                                repr(dpdx), repr(c), repr(L), repr(umax), repr(dref), str(fc), str(binary),
                                str(interval), repr(time_mean)], check=True, capture_output=True, text=True)
            pre = f"{name}__{k}__"
            for key, a in arrs.items():
                out[pre + "in_" + key] = a
            for key, a in means.items():
                out[pre + "in_" + key] = a
            vtk = os.path.join(work, "out", f"res{step:08d}.vtk")
            out[pre + "vtk"] = np.frombuffer(open(vtk, "rb").read(), dtype=np.uint8)
            out[pre + "data"] = np.frombuffer(open(os.path.join(work, "out", "data.dat"), "rb").read(), dtype=np.uint8)
            for key in ("rho", "u", "v", "w", "uMean", "vMean", "wMean"):
                out[pre + key] = np.fromfile(os.path.join(work, f"{key}.f32"), dtype=np.float32)
            rho_av, tm = open(os.path.join(work, "scalars.txt")).read().split()
            out[pre + "rho_av"] = np.array([np.float32(float(rho_av))])
            out[pre + "time_mean"] = np.array([np.float32(float(tm))])
            keep = [ln for ln in r.stdout.splitlines() if ln.startswith(("uAve:", "rhoMax:", "Cx:", "CxIBM:"))]
            out[pre + "console"] = np.frombuffer("\n".join(keep).encode(), dtype=np.uint8)
            out[pre + "spec"] = np.array([q, nx, ny, nz, step, fc, binary, interval])
            out[pre + "fspec"] = np.array([dpdx, c, L, umax, dref], dtype=np.float64)
            means = {key: out[pre + key].copy() for key in ("uMean", "vMean", "wMean")}
            time_mean = float(out[pre + "time_mean"][0])
        print(name, k, "vtk", out[pre + "vtk"].size, "bytes;", "\n  ".join(keep))


def main():
    out = {}
    for name, spec in CASES.items():
        run_case(name, spec, out)
    np.savez_compressed(os.path.join(HERE, "output_step.npz"), **out)


if __name__ == "__main__":
    main()
