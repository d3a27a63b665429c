"""Parity of the CUDA step with the reference (golden vectors) and with the CPU oracle.

Tolerances (FP32 populations, different operation order and FMA contraction):
  * rho and u after N steps: max |gpu - ref| <= 1e-5 * max |ref|  (the spec bar)
  * full population field vs the FP32 oracle: 1e-5 relative
  * FP16S storage: relative L2 velocity error vs the FP64 oracle <= 1e-3
  * integer work (link tables, cell classes): exact
"""
import os

import numpy as np
import pytest

from lbffs_gb300 import case as K
from parity_cases import REFERENCE_CASES, assert_fp32_parity, build, rel_err, rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def run_gpu(name, storage="fp32", steps=None, store_fields=2, c=None, run=None, special_kernel=-1, border_pulls=1):
    import lbffs_gb300 as L
    if c is None:
        c, run = build(name)
    lat = L.Lattice(c.nx, c.ny, c.nz, q=c.q, storage=storage, collision=run["collision"], sgs=run["sgs"],
                    wall=run["wall"], damping=run.get("damping", "wall"))
    lat.set_special_kernel(special_kernel)
    lat.set_border_pulls(border_pulls)
    lat.load_case(c)
    if "markers" in run:
        lat.set_markers(run["markers"])
        lat.set_motion(trans=run["motion"]["trans"], rot=(0, 0, 0), axis=(0, 0, 1), rot_omega=0.0)
    kw = run["kw"]
    lat.step(steps or run["steps"], dpdx=kw.get("dpdx", 0.0), les=kw.get("LES", 0.0),
             spz_width=kw.get("spzWidth", 0.1), store_fields=store_fields)
    lat.synchronize()
    return c, run, lat


def run_oracle(name, real="f32", steps=None):
    from oracle import ref as R
    c, run = build(name)
    o = R.OracleSolver(c, sgs=run["sgs"], wall=run["wall"], collision=run["collision"], real=real,
                       damping=run.get("damping", "wall"))
    if "markers" in run:
        o.set_ibm(run["markers"], *run["motion"]["trans"], rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), rot_omega=0.0)
    o.step(steps or run["steps"], **run["kw"])
    return o


@pytest.mark.parametrize("name", REFERENCE_CASES)
def test_gpu_fp32_matches_reference_golden(cuda_lib, name):
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    _, _, lat = run_gpu(name)
    rho, u, v, w = lat.macros()
    noise = float(g["noise_l2"])
    assert_fp32_parity(rho, np.stack([u, v, w]), g["rho"], np.stack([g["u"], g["v"], g["w"]]), noise)
    assert rel_l2(np.stack([u, v, w]), np.stack([g["u64"], g["v64"], g["w64"]])) < max(1e-5, 2.0 * noise)
    if "f" in g:
        assert rel_err(lat.download("f"), g["f"]) < 1e-5
    if "markers" in g:
        assert np.abs(lat.markers() - g["markers"]).max() < 1e-4


@pytest.mark.parametrize("name", REFERENCE_CASES)
def test_gpu_fp32_matches_oracle_fields(cuda_lib, oracle_built, name):
    c, run, lat = run_gpu(name)
    o = run_oracle(name)
    assert rel_err(lat.download("f"), o.f) < 1e-5
    fluid = c.solid == 0
    noise = float(np.load(os.path.join(GOLDEN, f"{name}.npz"))["noise_l2"])
    vel = np.stack([lat.download(k)[fluid] for k in ("u", "v", "w")])
    vel_o = np.stack([o.field(k)[fluid] for k in ("u", "v", "w")])
    assert_fp32_parity(lat.download("rho")[fluid], vel, o.field("rho")[fluid], vel_o, noise)
    tau_g, tau_o = lat.download("tau_sgs")[fluid], o.field("tauSGS")[fluid]
    if np.abs(tau_o).max() > 0:
        # tau_SGS ~ sqrt(|Pi_neq|) amplifies FP32 noise of the small non-equilibrium stress
        assert rel_l2(tau_g, tau_o) < max(1e-3, 100.0 * noise), rel_l2(tau_g, tau_o)
    else:
        assert np.abs(tau_g).max() == 0.0
    fw_o = np.stack([o.field("Fwx"), o.field("Fwy"), o.field("Fwz")])
    fw_g = np.stack([lat.download("fwx"), lat.download("fwy"), lat.download("fwz")])
    assert np.abs(fw_g - fw_o).max() <= max(1e-4, 10.0 * noise) * max(np.abs(fw_o).max(), 1e-6)
    s, so = lat.force_sum(), fw_o.astype(np.float64).sum(1)
    assert np.abs(s - so).max() <= max(1e-4, 10.0 * noise) * max(np.linalg.norm(so), 1e-6)


def _link_table(c):
    """(cell, mask) pairs of neiSolid && solid[upwind] from the reference's arrays (kernel.cl:1940-1943)."""
    cv, _ = K.lattice(c.q)
    s = c.solid.reshape(c.nz, c.ny, c.nx).astype(bool)
    masks = np.zeros(c.elements, np.uint32)
    for q in range(1, c.q):
        up = np.roll(s, shift=(int(cv[q, 2]), int(cv[q, 1]), int(cv[q, 0])), axis=(0, 1, 2)).ravel()
        masks |= ((c.nei_solid == 1) & (c.solid == 0) & up).astype(np.uint32) << np.uint32(q)
    cells = np.nonzero(masks)[0]
    return cells, masks[cells]


@pytest.mark.parametrize("name", ["cylinder_q19_bb", "cylinder2d_q19_ibb", "cylinder_q27_cumulant_les",
                                  "step_q19_les", "density_q19_dpdx"])
def test_link_table_bit_exact(cuda_lib, name):
    import lbffs_gb300 as L
    c, run = build(name)
    lat = L.Lattice(c.nx, c.ny, c.nz, q=c.q, collision=run["collision"], sgs=run["sgs"], wall=run["wall"])
    lat.load_case(c)
    cells, masks = lat.links()
    rc, rm = _link_table(c)
    assert np.array_equal(cells, rc) and np.array_equal(masks, rm)
    counts = lat.cell_counts()
    assert counts["fluid"] == int((c.solid == 0).sum()) and counts["link"] == len(rc)


def test_fp16s_velocity_error_vs_fp64_oracle(cuda_lib, oracle_built):
    c = K.make_case(24, 24, 24, 19, K.cavity_faces(0.05), nu=0.032)
    run = dict(sgs="smag", wall="bb", collision="rr", kw={})
    from oracle import ref as R
    o = R.OracleSolver(c, real="f64")
    o.step(300)
    _, u0, v0, w0 = o.macros()
    ref = np.stack([u0, v0, w0])
    out = {}
    for st in ("fp32", "fp16s", "bf16s"):
        _, _, lat = run_gpu(None, storage=st, steps=300, c=c, run=run)
        _, u, v, w = lat.macros()
        out[st] = float(np.linalg.norm(np.stack([u, v, w]) - ref) / np.linalg.norm(ref))
    print("velocity error vs FP64 oracle, 24^3 cavity, 300 steps:", out)
    assert out["fp32"] < 1e-5, out
    assert out["fp16s"] < 1e-3, out
    # BF16S (8 significand bits on f - w) does not meet the 1e-3 accuracy bar of the reduced-precision
    # storage; it is kept as a storage option below that bar, and this bound only guards it from
    # getting worse
    assert out["bf16s"] < 5e-2, out


@pytest.mark.parametrize("name", ["bluff_q27_les_ibm", "step_q19_les", "wallfn_q19", "bluff_q27_rr_les_ibm",
                                  "step_q27_rr_les", "step_q27_rr_vandriest", "cylinder_q27_rr_ibb_les_sponge"])
def test_fp16s_boundary_cases_vs_fp64_oracle(cuda_lib, oracle_built, name):
    """FP16S storage on the reduced bluff body (D3Q27, IBB, LES, IBM; cumulant and RR), the LES
    backward-facing step (D3Q19, and D3Q27 RR with either damping), the D3Q27 RR cylinder channel and the
    wall-function channel: relative L2 velocity error against the FP64 oracle <= 1e-3."""
    c, run = build(name)
    o = run_oracle(name, real="f64")
    fluid = c.solid == 0
    ref = np.stack([o.field(k)[fluid] for k in ("u", "v", "w")])
    _, _, lat = run_gpu(name, storage="fp16s")
    vel = np.stack([lat.download(k)[fluid] for k in ("u", "v", "w")])
    assert rel_l2(vel, ref) < 1e-3, rel_l2(vel, ref)


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
@pytest.mark.parametrize("name", ["cylinder2d_q19_ibb", "cylinder_q19_ibb_les_sponge", "cylinder_q19_bb", "mixed_q19",
                                  "density_q19_dpdx", "wallfn_q19", "step_q19_les", "step_q19_les_vandriest",
                                  "cavity_q19_wale", "ibm_q19"])
def test_boundary_kernel_mappings_agree_bitwise(cuda_lib, name, storage):
    """The boundary kernel with one thread per listed cell and with a lane group per cell (each lane
    reading its directions) computes the same bits: populations, macroscopic fields, eddy viscosity,
    wall force."""
    out = []
    for kind in (0, 1):
        _, _, lat = run_gpu(name, storage=storage, special_kernel=kind)
        out.append([lat.download(k) for k in ("f", "rho", "u", "v", "w", "tau_sgs", "fwx", "fwy", "fwz")])
        lat.close()
    for k, (x, y) in enumerate(zip(*out)):
        assert np.array_equal(x, y), (k, float(np.abs(x - y).max()))


def test_storage_modes_agree_with_each_other(cuda_lib):
    res = {}
    for st in ("fp32", "fp16s"):
        _, _, lat = run_gpu("cylinder_q19_ibb_les_sponge", storage=st)
        res[st] = lat.macros()
    assert rel_err(res["fp16s"][0], res["fp32"][0]) < 1e-3


def test_store_fields_does_not_change_populations(cuda_lib):
    _, _, a = run_gpu("cylinder_q19_ibb_les_sponge", store_fields=0)
    _, _, b = run_gpu("cylinder_q19_ibb_les_sponge", store_fields=2)
    assert np.array_equal(a.download("f"), b.download("f"))


def test_run_to_run_bitwise_deterministic(cuda_lib):
    _, _, a = run_gpu("cylinder_q27_cumulant_les")
    _, _, b = run_gpu("cylinder_q27_cumulant_les")
    assert np.array_equal(a.download("f"), b.download("f"))


@pytest.mark.parametrize("name", ["ibm_q19", "bluff_q27_les_ibm"])
def test_ibm_run_to_run_bitwise_deterministic(cuda_lib, name):
    """The IBM spread adds each marker's float-valued weighted force into an FP64 accumulator with
    atomics.  A double holds 53 significant bits and each float term 24, so the sum of one cell's terms
    is exact, and independent of the order in which the markers arrive, as long as those terms span
    fewer than 29 binary orders of magnitude, which they do on these cases."""
    _, _, a = run_gpu(name)
    _, _, b = run_gpu(name)
    assert np.array_equal(a.download("f"), b.download("f"))
    assert np.array_equal(a.markers(), b.markers())
    assert np.array_equal(a.download("gx"), b.download("gx"))


def test_fp64_mass_matches_oracle_and_is_conserved(cuda_lib, oracle_built):
    """FP64 mass reduction matches the FP64 oracle; over further steps the FP32 mass drift of the closed
    cavity stays within twice the FP32 oracle's own drift on the same case (the reference's FP32 path
    drifts by the same amount: FP32 rounding, not a conservation error)."""
    from oracle import ref as R
    c, run = build("cavity_q19")
    _, _, lat = run_gpu("cavity_q19", c=c, run=run)
    o = run_oracle("cavity_q19", real="f64")
    rho_o = o.macros()[0]
    assert abs(lat.mass() - rho_o.sum()) < 1e-6 * rho_o.sum()
    m0 = float(c.f.astype(np.float64).sum())
    lat.step(200)
    lat.synchronize()
    o32 = R.OracleSolver(c, real="f32")
    o32.step(run["steps"] + 200)
    drift_oracle = abs(float(o32.f.astype(np.float64).sum()) - m0) / m0
    drift_gpu = abs(lat.mass() - m0) / m0
    assert drift_gpu <= max(2.0 * drift_oracle, 2e-7), (drift_gpu, drift_oracle)


def test_ibm_markers_and_forcing_match_oracle(cuda_lib, oracle_built):
    c, run, lat = run_gpu("ibm_q19")
    o = run_oracle("ibm_q19")
    assert np.abs(lat.markers() - o.ibm_arrays["markers"].reshape(-1, 3)).max() < 1e-4
    g = np.stack([lat.download("gx"), lat.download("gy"), lat.download("gz")])
    go = np.stack([o.field("Gx"), o.field("Gy"), o.field("Gz")])
    assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max()
    assert rel_err(lat.download("f"), o.f) < 1e-5


def test_sinusoidal_marker_motion(cuda_lib, oracle_built):
    import lbffs_gb300 as L
    from oracle import ref as R
    c, run = build("ibm_q19")
    lat = L.Lattice(c.nx, c.ny, c.nz, q=19)
    lat.load_case(c)
    lat.set_markers(run["markers"])
    lat.set_motion(amp=(0.0, 2.0, 0.0), period=40.0, axis=(0, 0, 1))
    lat.step(25)
    lat.synchronize()
    o = R.OracleSolver(c, real="f32")
    o.set_ibm(run["markers"], axis=(0.0, 0.0, 1.0))
    o.set_motion(amp=(0.0, 2.0, 0.0), period=40.0)
    o.step(25)
    m = lat.markers()
    assert np.abs(m - o.ibm_arrays["markers"].reshape(-1, 3)).max() < 1e-4
    expect_dy = 2.0 * np.sin(2 * np.pi * 25 / 40.0)
    assert abs((m[:, 1] - run["markers"][:, 1]).mean() - expect_dy) < 1e-4
    assert rel_err(lat.download("f"), o.f) < 1e-5


def test_errors_are_status_codes(cuda_lib):
    import lbffs_gb300 as L
    lat = L.Lattice(8, 8, 8)
    with pytest.raises(L.LbffsError) as e:
        lat.upload("omega", np.ones(10, np.float32))
    assert e.value.code == L.E_ARG
    c = K.make_case(8, 8, 8, 19, K.cavity_faces(0.05))
    lat.load_case(c)
    b1 = c.boundary1.copy()
    b1[b1 == K.BOUNCEBACK] = 2  # no boundary code 2 exists (src/input.hpp:221-256)
    lat.upload("boundary1", b1)
    with pytest.raises(L.LbffsError) as e:
        lat.step(1)
    assert e.value.code == L.E_ARG


def test_divergence_sentinel_reports_nonfinite(cuda_lib):
    import lbffs_gb300 as L
    c = K.make_case(8, 8, 8, 19, K.cavity_faces(0.05))
    lat = L.Lattice(8, 8, 8)
    lat.load_case(c)
    f = c.f.copy()
    f[5 * c.elements + 3 * 64 + 3 * 8 + 3] = np.nan
    lat.upload("f", f)
    lat.step(2)
    with pytest.raises(L.LbffsError) as e:
        lat.synchronize()
    assert e.value.code == L.E_NONFINITE


def test_kernel_timing_counts_launches(cuda_lib):
    import lbffs_gb300 as L
    c = K.make_case(32, 32, 32, 19, K.cavity_faces(0.05))
    lat = L.Lattice(32, 32, 32)
    lat.load_case(c)
    lat.set_timing(True)
    lat.step(10)
    ms, n = lat.kernel_time("bulk")
    assert n == 10 and ms > 0
    ms, n = lat.kernel_time("special")
    assert n == 10


def test_large_cavity_mass_and_symmetry(cuda_lib):
    """Size-independent properties at 128^3: FP64 mass conservation of the closed cavity and the
    z-mirror symmetry of the lid-driven flow (lid velocity along x, walls symmetric in z)."""
    import lbffs_gb300 as L
    n = 128
    c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.032)
    lat = L.Lattice(n, n, n)
    lat.load_case(c)
    m0 = lat.mass()
    lat.step(200, store_fields=1)
    lat.synchronize()
    # the reference's FP32 path drifts 5e-9 per step on this case (1.0e-6 after 200 steps at 48^3)
    assert abs(lat.mass() - m0) < 2.0 * 5.1e-9 * 200 * m0
    u = lat.download("u").reshape(n, n, n)
    w = lat.download("w").reshape(n, n, n)
    assert np.abs(u - u[::-1]).max() < 1e-5 * np.abs(u).max()
    assert np.abs(w + w[::-1]).max() < 1e-5 * max(np.abs(u).max(), 1e-6)


@pytest.mark.parametrize("name", ["ellipsoid_q19", "ellipsoid_q27"])
def test_reference_voxelised_body_links_and_ibb(cuda_lib, oracle_built, name):
    """Geometry produced by the reference's own voxeliser (walls.hpp/stl.hpp): the device link table is
    bit-exact and the interpolated bounce-back run on it matches the oracle."""
    import lbffs_gb300 as L
    from oracle import ref as R
    g = np.load(os.path.join(GOLDEN, "setup_voxels.npz"))
    q, nx, ny, nz = (int(v) for v in g[f"{name}__shape"])
    # x / y walls as in the voxeliser run, the y-max wall moving (a lid) to drive flow past the body
    faces = {"nxMin": K.FaceBC(K.BOUNCEBACK, 0, 0), "nxMax": K.FaceBC(K.BOUNCEBACK, 0, 0),
             "nyMin": K.FaceBC(0, K.BOUNCEBACK, 0), "nyMax": K.FaceBC(0, K.FIXEDVELOCITY, 0, 0.05, 0, 0),
             "nzMin": K.FaceBC(), "nzMax": K.FaceBC()}
    c = K.make_case(nx, ny, nz, q, faces, nu=0.01, solid=g[f"{name}__solid"], sdf=g[f"{name}__sdf"])
    assert np.array_equal(c.nei_solid, g[f"{name}__nei_solid"])
    coll = "cumulant" if q == 27 else "rr"
    lat = L.Lattice(nx, ny, nz, q=q, collision=coll, wall="ibb")
    lat.load_case(c)
    cells, masks = lat.links()
    rc, rm = _link_table(c)
    assert len(rc) > 500 and np.array_equal(cells, rc) and np.array_equal(masks, rm)
    lat.step(20, les=1.0, store_fields=2)
    lat.synchronize()
    o = R.OracleSolver(c, sgs="smag", wall="ibb", collision=coll, real="f32")
    o.step(20, LES=1.0)
    assert rel_err(lat.download("f"), o.f) < 1e-5
    fw_o = np.stack([o.field("Fwx"), o.field("Fwy"), o.field("Fwz")]).astype(np.float64).sum(1)
    assert np.allclose(lat.force_sum(), fw_o, rtol=1e-4, atol=1e-6)
