"""GPU parity of the paths with no reference counterpart: the D3Q27 recursive-regularised collision and
the Van Driest near-wall damping (tests/parity_cases.py ORACLE_CASES).

The oracle's D3Q27 RR operator is pinned by tests/test_rr27_pins.py (D3Q19 limit, analytic Poiseuille,
shear-wave and Couette flows) and its Van Driest damping is a restatement of the reference's commented
block (D3Q19_opencl/kernel.cl:2178-2197).
Tolerances, as for the reference cases, with the case's FP32 round-off floor `noise`:
  * populations vs the FP32 oracle: max |gpu - oracle| <= 1e-5 * max |oracle|
  * rho, u vs the FP32 oracle and u vs the FP64 oracle: relative L2 <= max(1e-5, 2 * noise)
  * FP16S storage (the 24^3 D3Q27 RR cavity, 300 steps): relative L2 velocity error vs FP64 <= 1e-3
The floor is the larger of the FP32 oracle's own distance from the FP64 oracle on the case and the
reference's FP32-vs-FP64 distance on its matching reference case (TWIN below, from the golden
vectors): an FP32 implementation of a D3Q27 step lands anywhere within that floor, and the oracle's
FP32 run sits low in it (1.9e-6 on the mixed-face case, where the reference's own FP32 cumulant run
is 7.9e-6 from FP64).  Measured GPU distances from FP64: 3e-6 to 8.6e-6 without LES, 1.4e-5 on the
D3Q27 LES cases (the reference's FP32 run on its D3Q27 LES case: 1.6e-5).
"""
import os

import numpy as np
import pytest

from lbffs_gb300 import case as K
from parity_cases import ORACLE_CASES, assert_fp32_parity, build, rel_err, rel_l2
from test_gpu_parity import run_gpu, run_oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
# the reference case each oracle case mirrors (same lattice, boundaries and SGS setting)
TWIN = {"cavity_q27_rr": "cavity_q27_wale", "mixed_q27_rr": "mixed_q27_cumulant",
        "cylinder_q27_rr_ibb_les_sponge": "cylinder_q27_cumulant_les", "step_q27_rr_les": "cylinder_q27_cumulant_les",
        "step_q27_rr_vandriest": "cylinder_q27_cumulant_les", "step_q19_les_vandriest": "step_q19_les",
        "bluff_q27_rr_les_ibm": "bluff_q27_les_ibm"}


@pytest.mark.parametrize("name", ORACLE_CASES)
def test_gpu_matches_fp32_and_fp64_oracle(cuda_lib, oracle_built, name):
    c, run, lat = run_gpu(name)
    o32 = run_oracle(name, real="f32")
    o64 = run_oracle(name, real="f64")
    assert rel_err(lat.download("f"), o32.f) < 1e-5
    fluid = c.solid == 0
    vel = np.stack([lat.download(k)[fluid] for k in ("u", "v", "w")])
    vel32 = np.stack([o32.field(k)[fluid] for k in ("u", "v", "w")])
    vel64 = np.stack([o64.field(k)[fluid] for k in ("u", "v", "w")])
    noise_oracle = rel_l2(vel32, vel64)
    noise = max(noise_oracle, float(np.load(os.path.join(GOLDEN, f"{TWIN[name]}.npz"))["noise_l2"]))
    print(f"{name}: u vs FP32 oracle {rel_l2(vel, vel32):.3e}, vs FP64 {rel_l2(vel, vel64):.3e} (FP32 oracle vs FP64 "
          f"{noise_oracle:.3e}, floor {noise:.3e})")
    assert_fp32_parity(lat.download("rho")[fluid], vel, o32.field("rho")[fluid], vel32, noise)
    assert rel_l2(vel, vel64) < max(1e-5, 2.0 * noise), (rel_l2(vel, vel64), noise)
    tau_g, tau_o = lat.download("tau_sgs")[fluid], o64.field("tauSGS")[fluid]
    if np.abs(tau_o).max() > 0:
        assert rel_l2(tau_g, tau_o) < 1e-3, rel_l2(tau_g, tau_o)
    fw_o = np.stack([o64.field("Fwx"), o64.field("Fwy"), o64.field("Fwz")]).astype(np.float64).sum(1)
    assert np.abs(lat.force_sum() - fw_o).max() <= 1e-4 * max(np.linalg.norm(fw_o), 1e-6)


def test_fp16s_d3q27_rr_cavity_vs_fp64_oracle(cuda_lib, oracle_built):
    from oracle import ref as R
    c = K.make_case(24, 24, 24, 27, K.cavity_faces(0.05), nu=0.032)
    run = dict(sgs="smag", wall="ibb", collision="rr", kw={})
    o = R.OracleSolver(c, real="f64", collision="rr", wall="ibb")
    o.step(300)
    _, u0, v0, w0 = o.macros()
    ref = np.stack([u0, v0, w0])
    out = {}
    for st in ("fp32", "fp16s"):
        _, _, lat = run_gpu(None, storage=st, steps=300, c=c, run=run)
        _, u, v, w = lat.macros()
        out[st] = rel_l2(np.stack([u, v, w]), ref)
    assert out["fp32"] < 1e-5, out
    assert out["fp16s"] < 1e-3, out


def test_van_driest_changes_the_eddy_viscosity(cuda_lib):
    """The damping option reaches the kernels: the same step case with the reference's factor and with
    Van Driest damping gives different eddy viscosities near the walls, and no damping gives no smaller
    ones there."""
    c, run = build("step_q27_rr_les")
    res = {}
    for damp in ("wall", "vandriest", "none"):
        _, _, lat = run_gpu(None, c=c, run=dict(run, damping=damp))
        res[damp] = lat.download("tau_sgs")
    near = (c.sdf != K.SDF_NONE) & (c.sdf > 0) & (c.solid == 0)
    assert np.abs(res["vandriest"][near] - res["wall"][near]).max() > 1e-4 * np.abs(res["wall"]).max()
    assert np.all(res["none"][near] >= res["wall"][near] - 1e-7)
