"""The CPU oracle is pinned before it is trusted (CPU only).

* against golden vectors recorded from the reference's own kernels (tests/golden),
* against the reference compiled from source here (oracle/_ref) in FP64, where the
  restatement must agree to round-off after tens of steps.
"""
import os

import numpy as np
import pytest

from oracle import ref as R
from parity_cases import REFERENCE_CASES, assert_fp32_parity, build, rel_err, rel_l2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _oracle_run(name, real):
    c, run = build(name)
    o = R.OracleSolver(c, sgs=run["sgs"], wall=run["wall"], collision=run["collision"], real=real)
    if "markers" in run:
        o.set_ibm(run["markers"], *run["motion"]["trans"], rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), rot_omega=0.0)
    o.step(run["steps"], **run["kw"])
    return c, run, o


@pytest.mark.parametrize("name", REFERENCE_CASES)
def test_oracle_fp32_matches_reference_golden(oracle_built, name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    _, _, o = _oracle_run(name, "f32")
    rho, u, v, w = o.macros()
    noise = float(g["noise_l2"])
    assert_fp32_parity(rho, np.stack([u, v, w]), g["rho"], np.stack([g["u"], g["v"], g["w"]]), noise)
    # as close to the reference's FP64 answer as the reference's FP32 run is
    assert rel_l2(np.stack([u, v, w]), np.stack([g["u64"], g["v64"], g["w64"]])) < max(1e-5, 2.0 * noise)


@pytest.mark.parametrize("name", REFERENCE_CASES)
def test_oracle_fp64_matches_reference_fp64(oracle_built, name):
    c, run = build(name)
    if not R.available(c.q, run["sgs"], run["wall"], "f64"):
        pytest.skip("reference kernels not compiled here (oracle/_ref)")
    _, _, o = _oracle_run(name, "f64")
    r = R.RefSolver(c, sgs=run["sgs"], wall=run["wall"], real="f64")
    if "markers" in run:
        r.set_ibm(run["markers"], *run["motion"]["trans"], rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), rot_omega=0.0)
    r.step(run["steps"], **run["kw"])
    # the reference's FP64 build keeps single-rounded float literals (weights 1.f/18.f ...), ~1e-8 relative
    assert rel_err(o.f, r.f) < 1e-6
    ro, uo, vo, wo = o.macros()
    rr, ur, vr, wr = r.macros()
    assert rel_err(np.stack([uo, vo, wo]), np.stack([ur, vr, wr])) < 1e-6


def test_oracle_fp64_vs_fp32_drift_small(oracle_built):
    _, _, o32 = _oracle_run("cavity_q19", "f32")
    _, _, o64 = _oracle_run("cavity_q19", "f64")
    assert rel_err(o32.f, o64.f) < 1e-5


def test_oracle_detects_planted_bc_mistake(oracle_built):
    """A mistake planted in the oracle's inputs (lid velocity sign) must break the golden comparison."""
    g = np.load(os.path.join(GOLDEN, "cavity_q19.npz"))
    c, run = build("cavity_q19")
    c.u0 = np.where(c.u0 != 0, -c.u0, c.u0).astype(np.float32)
    o = R.OracleSolver(c, sgs=run["sgs"], wall=run["wall"], real="f32")
    o.step(run["steps"])
    _, u, v, w = o.macros()
    assert rel_err(np.stack([u, v, w]), np.stack([g["u"], g["v"], g["w"]])) > 0.5
