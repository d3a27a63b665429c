"""Small, seeded cases shared by the golden-vector generator and the parity tests.

Each case is built with :mod:`lbffs_gb300.case` / :mod:`lbffs_gb300.geometry`
exactly as the reference driver would build it (ns.cpp setup), so the same
arrays can be fed to the reference compiled from source (``oracle/_ref``), to
the CPU restatement (``oracle/``) and to the CUDA library.
"""
from __future__ import annotations

import numpy as np

from lbffs_gb300.case import (BOUNCEBACK, CYCLIC, FIXEDDENSITY, FIXEDVELOCITY, OUTLET, SYMMETRY, WALLFUNCTION,
                              FaceBC, cavity_faces, channel_faces, make_case)
from lbffs_gb300.geometry import backward_step, cylinder_markers, cylinder_z, ellipsoid


def _mixed_faces():
    return {"nxMin": FaceBC(FIXEDVELOCITY, 0, 0, 0.04, 0.01, 0.0), "nxMax": FaceBC(OUTLET, 0, 0),
            "nyMin": FaceBC(0, SYMMETRY, 0), "nyMax": FaceBC(0, FIXEDVELOCITY, 0, 0.03, 0.0, 0.0),
            "nzMin": FaceBC(0, 0, SYMMETRY), "nzMax": FaceBC(0, 0, BOUNCEBACK)}


def _density_faces():
    f = channel_faces(0.05, top_bottom=BOUNCEBACK, z_periodic=False)
    f["nxMax"] = FaceBC(FIXEDDENSITY, CYCLIC, CYCLIC)
    return f


def _wallfn_faces():
    """Channel whose y faces are WallFunction walls (code 7), z periodic."""
    f = channel_faces(0.05, top_bottom=WALLFUNCTION, z_periodic=True)
    return f


def build(name):
    """Return (case, run) where run holds the solver selections and step keyword arguments."""
    if name == "cavity_q19":
        c = make_case(12, 12, 12, 19, cavity_faces(0.05), nu=0.032)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=60, kw={})
    if name == "cavity_q19_les":
        c = make_case(12, 12, 12, 19, cavity_faces(0.08), nu=0.002)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw=dict(LES=1.0))
    if name == "cavity_q19_wale":
        c = make_case(12, 12, 12, 19, cavity_faces(0.05), nu=0.01)
        return c, dict(sgs="wale", wall="bb", collision="rr", steps=40, kw={})
    if name == "cylinder_q19_ibb_les_sponge":
        solid, sdf = cylinder_z(32, 20, 6, 10.3, 9.8, 3.6)
        c = make_case(32, 20, 6, 19, channel_faces(0.05), nu=0.004, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=40, kw=dict(LES=1.0, spzWidth=0.2))
    if name == "cylinder_q19_bb":
        solid, sdf = cylinder_z(32, 20, 6, 10.3, 9.8, 3.6)
        c = make_case(32, 20, 6, 19, channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw={})
    if name == "cylinder2d_q19_ibb":
        solid, sdf = cylinder_z(40, 24, 1, 12.4, 11.7, 4.3)
        c = make_case(40, 24, 1, 19, channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=40, kw={})
    if name == "mixed_q19":
        c = make_case(16, 14, 12, 19, _mixed_faces(), nu=0.02)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw={})
    if name == "density_q19_dpdx":
        solid, sdf = cylinder_z(28, 18, 8, 9.0, 8.6, 3.1)
        c = make_case(28, 18, 8, 19, _density_faces(), nu=0.02, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw=dict(dpdx=1e-5))
    if name == "step_q19_les":
        solid, sdf = backward_step(40, 16, 8, 12, 6)
        f = channel_faces(0.06, top_bottom=BOUNCEBACK, z_periodic=True)
        c = make_case(40, 16, 8, 19, f, nu=0.001, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw=dict(LES=1.0, spzWidth=0.25))
    if name == "mixed_q27_cumulant":
        c = make_case(16, 14, 12, 27, _mixed_faces(), nu=0.02)
        return c, dict(sgs="smag", wall="ibb", collision="cumulant", steps=30, kw={})
    if name == "cylinder_q27_cumulant_les":
        solid, sdf = cylinder_z(28, 18, 8, 9.2, 8.7, 3.3)
        c = make_case(28, 18, 8, 27, channel_faces(0.05), nu=0.003, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="ibb", collision="cumulant", steps=30, kw=dict(LES=1.0))
    if name == "cavity_q27_wale":
        c = make_case(12, 12, 12, 27, cavity_faces(0.05), nu=0.01)
        return c, dict(sgs="wale", wall="ibb", collision="cumulant", steps=30, kw={})
    if name == "ibm_q19":
        c = make_case(32, 20, 6, 19, channel_faces(0.04), nu=0.02)
        m = cylinder_markers(24, 11.3, 9.7, 2.4, 3.2)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=30, kw={}, markers=m,
                       motion=dict(trans=(0.01, 0.0, 0.0)))
    if name == "bluff_q27_les_ibm":
        # the bluff-body configuration at reduced size: D3Q27, an ellipsoid body with interpolated
        # bounce-back, LES, and an IBM cylinder upstream (two marker rings, translating)
        solid, sdf = ellipsoid(48, 20, 20, (26.3, 9.8, 10.2), (9.0, 4.2, 4.4))
        c = make_case(48, 20, 20, 27, channel_faces(0.05), nu=0.002, solid=solid, sdf=sdf)
        m = np.concatenate([cylinder_markers(16, 8.2, 9.6, 9.5 + z, 2.5) for z in range(2)])
        return c, dict(sgs="smag", wall="ibb", collision="cumulant", steps=30, kw=dict(LES=1.0), markers=m,
                       motion=dict(trans=(0.0, 0.004, 0.0)))
    if name == "wallfn_q19":
        c = make_case(32, 16, 6, 19, _wallfn_faces(), nu=0.004)
        return c, dict(sgs="smag", wall="bb", collision="rr", steps=40, kw={})
    if name == "wallfn_q27":
        c = make_case(28, 14, 6, 27, _wallfn_faces(), nu=0.004)
        return c, dict(sgs="smag", wall="ibb", collision="cumulant", steps=30, kw={})
    # ---- D3Q27 recursive regularised collision and Van Driest damping: no reference counterpart, so
    # these cases are checked against the oracle (FP32 and FP64) only ----
    if name == "cavity_q27_rr":
        c = make_case(12, 12, 12, 27, cavity_faces(0.05), nu=0.032)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=60, kw={})
    if name == "mixed_q27_rr":
        c = make_case(16, 14, 12, 27, _mixed_faces(), nu=0.02)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=30, kw={})
    if name == "cylinder_q27_rr_ibb_les_sponge":
        solid, sdf = cylinder_z(28, 18, 8, 9.2, 8.7, 3.3)
        c = make_case(28, 18, 8, 27, channel_faces(0.05), nu=0.003, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=30, kw=dict(LES=1.0, spzWidth=0.2))
    if name == "step_q27_rr_les":
        # the backward-facing step at reduced size: walls top and bottom, z periodic, inlet 0.06
        solid, sdf = backward_step(40, 16, 8, 12, 6)
        f = channel_faces(0.06, top_bottom=BOUNCEBACK, z_periodic=True)
        c = make_case(40, 16, 8, 27, f, nu=0.001, solid=solid, sdf=sdf)
        return c, dict(sgs="smag", wall="ibb", collision="rr", steps=30, kw=dict(LES=1.0, spzWidth=0.25))
    if name == "step_q27_rr_vandriest":
        c, run = build("step_q27_rr_les")
        run["damping"] = "vandriest"
        return c, run
    if name == "step_q19_les_vandriest":
        c, run = build("step_q19_les")
        run["damping"] = "vandriest"
        return c, run
    if name == "bluff_q27_rr_les_ibm":
        c, run = build("bluff_q27_les_ibm")
        run["collision"] = "rr"
        return c, run
    raise KeyError(name)


# cases the reference itself can run (golden vectors are recorded from it)
REFERENCE_CASES = ["cavity_q19", "cavity_q19_les", "cavity_q19_wale", "cylinder_q19_ibb_les_sponge", "cylinder_q19_bb",
                   "cylinder2d_q19_ibb", "mixed_q19", "density_q19_dpdx", "step_q19_les", "mixed_q27_cumulant",
                   "cylinder_q27_cumulant_les", "cavity_q27_wale", "ibm_q19", "wallfn_q19", "wallfn_q27",
                   "bluff_q27_les_ibm"]


# cases with no reference counterpart (D3Q27 RR, Van Driest damping): checked against the oracle in
# FP32 and FP64
ORACLE_CASES = ["cavity_q27_rr", "mixed_q27_rr", "cylinder_q27_rr_ibb_les_sponge", "step_q27_rr_les",
                "step_q27_rr_vandriest", "step_q19_les_vandriest", "bluff_q27_rr_les_ibm"]


def rel_err(a, b):
    """max |a - b| / max |b| over the array."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2 over the array."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


# FP32 parity bar for rho and u after N steps: relative L2 <= 1e-5 over the field (the norm the
# storage-precision bar uses too), with a max-norm guard that catches localised mistakes.  Where
# the reference's own FP32 run is farther than that from its FP64 run (``noise``, recorded with
# the golden vectors: LES / WALE cases at low viscosity), the bar is twice that round-off floor.
L2_TOL = 1e-5
MAX_TOL = 5e-5


def assert_fp32_parity(rho, vel, rho_ref, vel_ref, noise=0.0):
    l2_tol = max(L2_TOL, 2.0 * noise)
    max_tol = max(MAX_TOL, 10.0 * noise)
    assert rel_err(rho, rho_ref) < 1e-5, ("rho", rel_err(rho, rho_ref))
    assert rel_l2(vel, vel_ref) < l2_tol, ("u L2", rel_l2(vel, vel_ref), l2_tol)
    assert rel_err(vel, vel_ref) < max_tol, ("u max", rel_err(vel, vel_ref), max_tol)
