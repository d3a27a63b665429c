"""The face streaming of every face kind against the FP32 oracle, cell by cell, and the border-pull
modes against the ghost fill, bit for bit.

A border cell pulls across the grid's edge what the reference's face streaming gives it (upwindID_B +
reflectOrMirrorQ, D3Q19 kernel.cl:114-575, D3Q27 kernel.cl:1133-1146): the periodic image across a
Cyclic face, the cell's own missing direction across a wall.  Where every face carries one code per
axis the step reads those values where they lie (mode 1: inlet / outlet x faces; mode 2: bulk cells
pull across Cyclic x faces from per-context plane bases; mode 3: bulk cells on x faces without a
Cyclic code write the ghost slots they pull from next step themselves); otherwise, and with
lbffs_set_border_pulls(ctx, 0), from the ghost layer filled before each step.  These cases put bulk
cells on every face kind the bulk kernels keep (Cyclic, BounceBack, Symmetry), with rows wider than
one warp (a thread's two cells 32 apart, or adjacent for 2-byte storage, meet an x face in either
lane) and a seeded perturbation of every population so that each pull is seen in the result.
Tolerances: FP32 storage within 1e-5 of the largest population (the parity bar of the other cases);
FP16S storage within 2e-5 absolute (its rounding of the 2^15-scaled deviation is about 1e-6 here).
"""
import numpy as np
import pytest

from lbffs_gb300 import case as K

pytestmark = pytest.mark.gpu


def _faces(kind, nz):
    if kind == "periodic_x":
        f = {"nyMin": K.FaceBC(K.CYCLIC, K.BOUNCEBACK, K.CYCLIC),
             "nyMax": K.FaceBC(K.CYCLIC, K.FIXEDVELOCITY, K.CYCLIC, 0.05, 0.0, 0.0)}
    elif kind == "walls_x":
        f = {"nxMin": K.FaceBC(K.BOUNCEBACK, K.CYCLIC, K.CYCLIC), "nxMax": K.FaceBC(K.BOUNCEBACK, K.CYCLIC, K.CYCLIC),
             "nyMin": K.FaceBC(K.CYCLIC, K.SYMMETRY, K.CYCLIC), "nyMax": K.FaceBC(K.CYCLIC, K.BOUNCEBACK, K.CYCLIC)}
    elif kind == "channel_x":  # border pulls: inlet and outlet x faces, y / z walls of both kinds
        f = {"nxMin": K.FaceBC(K.FIXEDVELOCITY, K.CYCLIC, K.CYCLIC, 0.05, 0.0, 0.0),
             "nxMax": K.FaceBC(K.OUTLET, K.CYCLIC, K.CYCLIC),
             "nyMin": K.FaceBC(K.CYCLIC, K.SYMMETRY, K.CYCLIC), "nyMax": K.FaceBC(K.CYCLIC, K.BOUNCEBACK, K.CYCLIC)}
    else:  # symmetry_x
        f = {"nxMin": K.FaceBC(K.SYMMETRY, K.CYCLIC, K.CYCLIC), "nxMax": K.FaceBC(K.SYMMETRY, K.CYCLIC, K.CYCLIC),
             "nyMin": K.FaceBC(K.CYCLIC, K.BOUNCEBACK, K.CYCLIC), "nyMax": K.FaceBC(K.CYCLIC, K.SYMMETRY, K.CYCLIC)}
    if nz > 1:
        f["nzMin"] = K.FaceBC(K.CYCLIC, K.CYCLIC, K.BOUNCEBACK)
        f["nzMax"] = K.FaceBC(K.CYCLIC, K.CYCLIC, K.SYMMETRY)
    return f


def _case(q, kind, nx, nz, seed):
    c = K.make_case(nx, 12, nz, q, _faces(kind, nz), nu=0.02)
    rng = np.random.default_rng(seed)
    c.f = (c.f + 2e-3 * rng.standard_normal(c.f.shape)).astype(np.float32)
    return c


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("kind,nx,nz", [("periodic_x", 72, 1), ("periodic_x", 33, 5), ("walls_x", 40, 4),
                                        ("symmetry_x", 65, 3), ("channel_x", 72, 1), ("channel_x", 40, 6)])
def test_border_pulls_match_oracle(cuda_lib, oracle_built, storage, q, kind, nx, nz):
    import lbffs_gb300 as L
    from oracle import ref as R
    c = _case(q, kind, nx, nz, seed=nx * 100 + nz)
    for steps in (1, 4):
        lat = L.Lattice(c.nx, c.ny, c.nz, q=q, storage=storage, collision="rr", sgs="smag", wall="bb")
        lat.load_case(c)
        lat.step(steps)
        lat.synchronize()
        f = lat.download("f").reshape(q, nz, c.ny, nx)
        o = R.OracleSolver(c, sgs="smag", wall="bb", collision="rr", real="f32")
        o.step(steps)
        g = o.f.reshape(q, nz, c.ny, nx)
        d = np.abs(f - g)
        tol = 1e-5 * np.abs(g).max() if storage == "fp32" else 2e-5
        bad = np.argwhere(d > tol)
        assert len(bad) == 0, (steps, float(d.max()), sorted(set(bad[:, 3].tolist()))[:8])


def _mode_case(q, kind, nx, nz):
    if kind == "cavity":
        faces = K.cavity_faces(0.05)
    elif kind == "channel":
        faces = K.channel_faces(0.05)
    else:
        faces = _faces(kind.replace("_solid", ""), nz)
    solid = None
    if kind.endswith("_solid"):
        # solid blocks on both x faces: link cells of the boundary kernel beside bulk cells there
        s = np.zeros((nz, 12, nx), np.uint8)
        s[1:3, 3:6, 0:3] = 1
        s[2:4, 6:9, nx - 2:] = 1
        solid = s.ravel()
    c = K.make_case(nx, 12, nz, q, faces, nu=0.02, solid=solid)
    rng = np.random.default_rng(nx + 7 * nz + q)
    c.f = (c.f + 2e-3 * rng.standard_normal(c.f.shape)).astype(np.float32)
    return c


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
@pytest.mark.parametrize("q,collision,sgs,les", [(19, "rr", "smag", 0.0), (19, "rr", "smag", 0.12),
                                                 (19, "rr", "wale", 0.0), (27, "rr", "smag", 0.12),
                                                 (27, "cumulant", "smag", 0.0)])
@pytest.mark.parametrize("kind,nx,nz", [("cavity", 37, 6), ("cavity", 301, 3), ("walls_x", 64, 4),
                                        ("symmetry_x", 33, 3), ("periodic_x", 70, 5), ("walls_x_solid", 45, 5),
                                        ("channel", 40, 4), ("walls_x", 40, 1)])
def _expected_halos(kind, q, storage, nz, steps):
    """Ghost fills a run of `steps` steps launches: none where the lattice pulls across all its faces
    (inlet / outlet x faces; Cyclic x faces where that kernel is built), one where the x-face cells
    write their own ghost slots (x faces without a Cyclic code: the fill before the first step), one
    per step otherwise (D3Q27 2-byte storage with Cyclic x faces; a 2D grid with wall-coded z faces,
    which these cases do not have: their 2D grids leave the z faces Cyclic)."""
    if kind == "channel":
        return 0
    if kind == "periodic_x":
        return 0 if (q == 19 or storage == "fp32") else steps
    return 1


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
@pytest.mark.parametrize("q,collision,sgs,les", [(19, "rr", "smag", 0.0), (19, "rr", "smag", 0.12),
                                                 (19, "rr", "wale", 0.0), (27, "rr", "smag", 0.12),
                                                 (27, "rr", "smag", 0.0), (27, "cumulant", "smag", 0.0)])
@pytest.mark.parametrize("kind,nx,nz", [("cavity", 37, 6), ("cavity", 301, 3), ("walls_x", 64, 4),
                                        ("symmetry_x", 33, 3), ("periodic_x", 70, 5), ("walls_x_solid", 45, 5),
                                        ("channel", 40, 4), ("walls_x", 40, 1)])
def test_pull_modes_agree_bitwise(cuda_lib, storage, q, collision, sgs, les, kind, nx, nz):
    """Reading every population that crosses the grid's border where the face streaming takes it gives
    the bits of reading it from a ghost layer filled before every step: populations and macroscopic
    fields after 5 steps.  Bulk cells lie on the x faces here (cavity, walls, symmetry, periodic x;
    odd row lengths and a second row tile end on an x face in either cell of a pair), beside
    boundary-kernel cells (the solid blocks' links, the lid), or only boundary-kernel cells do (the
    channel's inlet and outlet); the 2D grid has Cyclic z faces."""
    import lbffs_gb300 as L
    c = _mode_case(q, kind, nx, nz)
    out, halos = [], []
    for on in (1, 0):
        lat = L.Lattice(c.nx, c.ny, c.nz, q=q, storage=storage, collision=collision, sgs=sgs)
        lat.set_border_pulls(on)
        lat.set_timing(True)
        lat.load_case(c)
        lat.step(5, les=les)
        lat.synchronize()
        halos.append(lat.kernel_time("halo")[1])
        out.append([lat.download(k) for k in ("f", "rho", "u", "v", "w")])
        lat.close()
    assert halos[1] == 5
    assert halos[0] == _expected_halos(kind, q, storage, nz, 5)
    for k, (x, y) in enumerate(zip(*out)):
        assert np.array_equal(x, y), (k, float(np.abs(x - y).max()))


@pytest.mark.parametrize("storage", ["fp32", "fp16s"])
@pytest.mark.parametrize("q", [19, 27])
def test_ghost_slots_follow_state_changes(cuda_lib, storage, q):
    """Where x-face cells write their own ghost slots, every change of the populations from outside a
    step (an upload, a rest state, a switch of the pull setting) makes the next step fill the ghost
    layer first: a run interrupted by each of them gives the bits of the ghost-layer run."""
    import lbffs_gb300 as L
    c = _mode_case(q, "cavity", 45, 5)
    rng = np.random.default_rng(5)
    f2 = (c.f + 1e-3 * rng.standard_normal(c.f.shape)).astype(np.float32)
    out, halos = [], []
    for on in (1, 0):
        lat = L.Lattice(c.nx, c.ny, c.nz, q=q, storage=storage)
        lat.set_border_pulls(on)
        lat.set_timing(True)
        lat.load_case(c)
        lat.step(3)
        lat.upload("f", f2)
        lat.step(2)
        lat.set_border_pulls(on)
        lat.step(2)
        lat.init_rest()
        lat.step(2)
        lat.synchronize()
        halos.append(lat.kernel_time("halo")[1])
        out.append([lat.download(k) for k in ("f", "rho", "u", "v", "w")])
        lat.close()
    assert halos == [4, 9]
    for k, (x, y) in enumerate(zip(*out)):
        assert np.array_equal(x, y), (k, float(np.abs(x - y).max()))


@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("kind,nx,nz,storage", [("channel", 40, 6, "fp32"), ("channel", 40, 6, "fp16s"),
                                                ("periodic_x", 44, 6, "fp32"), ("cavity", 36, 6, "fp32"),
                                                ("cavity", 36, 6, "bf16s")])
def test_pull_modes_with_ibm_forcing_agree_bitwise(cuda_lib, q, kind, nx, nz, storage):
    """The IBM forcing pass changes populations after the step.  Reading across the border where the
    face streaming takes each population (inlet / outlet or Cyclic x faces) sees them as the ghost fill
    does: bitwise the ghost-layer run, with no fill.  Where the x-face cells would write their own ghost
    slots (the cavity) they would do so before the pass, so with markers that lattice fills the ghost
    layer before every step."""
    import lbffs_gb300 as L
    from lbffs_gb300.geometry import cylinder_markers
    c = _mode_case(q, kind, nx, nz)
    markers = cylinder_markers(24, nx * 0.4, 6.0, nz / 2.0, 2.5)
    out, halos = [], []
    for on in (1, 0):
        lat = L.Lattice(c.nx, c.ny, c.nz, q=q, storage=storage)
        lat.set_border_pulls(on)
        lat.set_timing(True)
        lat.load_case(c)
        lat.set_markers(markers)
        lat.set_motion(trans=(0.01, 0.0, 0.0), rot=(0, 0, 0), axis=(0, 0, 1), rot_omega=0.0)
        lat.step(6)
        lat.synchronize()
        halos.append(lat.kernel_time("halo")[1])
        out.append([lat.download(k) for k in ("f", "rho", "u", "v", "w")])
        lat.close()
    assert halos == [6 if kind == "cavity" else 0, 6]
    for k, (x, y) in enumerate(zip(*out)):
        assert np.array_equal(x, y), (k, float(np.abs(x - y).max()))
