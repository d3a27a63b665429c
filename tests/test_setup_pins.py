"""Host-side case setup matches the reference's own host code bit for bit (CPU only).

Golden vectors come from src/setBoundaryConditions.hpp and src/walls.hpp / src/stl.hpp
compiled from the reference sources (tests/golden/make_golden_setup.py).
"""
import os
import sys

import numpy as np
import pytest

from lbffs_gb300 import case as K

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_golden_setup as MG  # noqa: E402


@pytest.mark.parametrize("name", sorted(MG.FACE_SETS))
@pytest.mark.parametrize("grid", MG.FACE_GRIDS)
def test_face_arrays_bit_exact(name, grid):
    g = np.load(os.path.join(GOLDEN, "setup_faces.npz"))
    nx, ny, nz = grid
    faces = {fn: K.FaceBC(*fs) for fn, fs in zip(K.FACES, MG.FACE_SETS[name])}
    got = dict(zip(("boundary", "boundary1", "boundary2", "boundary3", "u0", "v0", "w0"),
                   K.face_arrays(nx, ny, nz, faces)))
    key = f"{name}_{nx}x{ny}x{nz}"
    for fld, arr in got.items():
        ref = g[f"{key}__{fld}"]
        assert arr.dtype == ref.dtype and np.array_equal(arr.view(np.uint8), ref.view(np.uint8)), (key, fld)


@pytest.mark.parametrize("name", sorted(MG.VOXEL_CASES))
def test_nei_solid_bit_exact(name):
    g = np.load(os.path.join(GOLDEN, "setup_voxels.npz"))
    q, nx, ny, nz = (int(v) for v in g[f"{name}__shape"])
    ns = K.nei_solid(g[f"{name}__solid"], nx, ny, nz, q)
    assert np.array_equal(ns, g[f"{name}__nei_solid"])
    assert g[f"{name}__solid"].sum() > 1000  # the mesh really voxelised


def test_equilibrium_initialisation_matches_golden_cavity():
    """initialization.hpp: f = feq(rho0, uIni) -- the cavity golden run starts from it."""
    c = K.make_case(12, 12, 12, 19, K.cavity_faces(0.05), nu=0.032)
    _, w = K.lattice(19)
    assert np.array_equal(c.f.reshape(19, -1)[:, 0], w)
