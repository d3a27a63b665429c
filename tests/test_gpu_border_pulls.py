"""The face streaming of every face kind against the FP32 oracle, cell by cell, in both pull modes.

A border cell pulls across the grid's edge what the reference's face streaming gives it (upwindID_B +
reflectOrMirrorQ, D3Q19 kernel.cl:114-575, D3Q27 kernel.cl:1133-1146): the periodic image across a
Cyclic face, the cell's own missing direction across a wall.  A lattice whose two x faces are
boundary-kernel faces (inlet / outlet) reads those values where they lie (border pulls: bulk rows on a
y / z face cross it by the row's border); any other lattice reads them from the ghost layer filled
before each step.  These cases put bulk cells on every face kind the bulk kernels keep (Cyclic,
BounceBack, Symmetry), with rows wider than one warp (a thread's two cells 32 apart, or adjacent for
2-byte storage, meet an x face in either lane) and a seeded perturbation of every population so that
each pull is seen in the result.
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
