"""Record golden vectors from the reference's own step kernels (run here, on the CPU).

For every case in ``tests/parity_cases.REFERENCE_CASES`` the reference
``k_streamingCollision`` (compiled from D3Q19_opencl/kernel.cl or
D3Q27_opencl/kernel.cl by ``oracle/build_ref.py``) advances the case in FP32 and
the macroscopic fields computed from the final populations (write.hpp's host
``cal_rhoUVW``) are saved, with the STL-link force sum.  The same case is also run in the reference's FP64
build; its velocity and the FP32-vs-FP64 distance of the reference itself
(``noise_l2``, the FP32 round-off floor of the case) are stored alongside.  The recipe needs the
reference checkout, so it runs in the build container; the .npz files it writes
are committed and travel with the tests.

usage: python tests/golden/make_golden.py [case ...]   (default: every case)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.ref import RefSolver  # noqa: E402
from parity_cases import REFERENCE_CASES, build  # noqa: E402


def main(names=None):
    for name in names or REFERENCE_CASES:
        c, run = build(name)
        r = RefSolver(c, sgs=run["sgs"], wall=run["wall"], real="f32", nthreads=1)
        if "markers" in run:
            r.set_ibm(run["markers"], *run["motion"]["trans"], rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0),
                      rot_omega=0.0)
        r.step(run["steps"], **run["kw"])
        rho, u, v, w = r.macros()
        # the same run in the reference's FP64 build: the exact answer the FP32 results are measured against
        r64 = RefSolver(c, sgs=run["sgs"], wall=run["wall"], real="f64", nthreads=1)
        if "markers" in run:
            r64.set_ibm(run["markers"], *run["motion"]["trans"], rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0),
                        rot_omega=0.0)
        r64.step(run["steps"], **run["kw"])
        _, u64, v64, w64 = r64.macros()
        vel, vel64 = np.stack([u, v, w]), np.stack([u64, v64, w64])
        noise = float(np.linalg.norm(vel - vel64) / np.linalg.norm(vel64))
        out = dict(rho=rho.astype(np.float32), u=u.astype(np.float32), v=v.astype(np.float32),
                   w=w.astype(np.float32), steps=run["steps"], u64=u64, v64=v64, w64=w64, noise_l2=noise,
                   fw_sum=np.array([r.field("Fwx").astype(np.float64).sum(), r.field("Fwy").astype(np.float64).sum(),
                                    r.field("Fwz").astype(np.float64).sum()]))
        if name == "cavity_q19":
            out["f"] = r.f.astype(np.float32)
        if "markers" in run:
            out["markers"] = r.ibm_arrays["markers"].reshape(-1, 3).astype(np.float32)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(f"{name}: {c.nx}x{c.ny}x{c.nz} q{c.q} steps={run['steps']} fp32 noise {noise:.2e}")


if __name__ == "__main__":
    main(sys.argv[1:])
