"""Device voxelisation (lbffs_voxelize) against the reference's own host voxeliser: solid and
neiSolid bit for bit on the fixtures the reference wrote (src/walls.hpp setSolid / setNeiSolid run
on seeded ellipsoid meshes, including an inverted fluid/solid case and a 6240-triangle mesh)."""
import os

import numpy as np
import pytest

from lbffs_gb300 import geometry as G

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# the meshes of tests/golden/make_golden_setup.py
MESHES = {
    "ellipsoid_q19": lambda: G.ellipsoid_mesh(7, 18, 36, (19.3, 15.6, 14.8), (11.0, 8.0, 7.5)),
    "ellipsoid_q27": lambda: G.ellipsoid_mesh(11, 18, 36, (20.1, 16.2, 15.1), (12.0, 9.0, 8.0)),
    "ellipsoid_big_q19": lambda: G.ellipsoid_mesh(23, 40, 80, (47.7, 39.2, 35.6), (30.0, 22.0, 20.5), noise=0.05),
    "ellipsoid_inv_q19": lambda: G.ellipsoid_mesh(31, 18, 36, (19.1, 15.9, 14.6), (13.0, 10.0, 9.0)),
}


def stl_vertices(tris):
    """Vertices as the reference reads them from write_ascii_stl's text (std::stof of each field)."""
    return np.array([[[np.float32(f"{x:.6e}") for x in v] for v in t] for t in tris], dtype=np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MESHES))
def test_voxelize_matches_reference_voxeliser(cuda_lib, name):
    import lbffs_gb300 as L
    g = np.load(os.path.join(GOLDEN, "setup_voxels.npz"))
    q, nx, ny, nz = (int(v) for v in g[f"{name}__shape"])
    invert = bool(int(g[f"{name}__invert"][0]))
    lat = L.Lattice(nx, ny, nz, q=q, wall="ibb" if q == 27 else "bb")
    lat.voxelize(stl_vertices(MESHES[name]()), invert=invert)
    solid = lat.download("solid")
    nei = lat.download("nei_solid")
    lat.close()
    assert np.array_equal(solid, g[f"{name}__solid"]), (name, int((solid != g[f"{name}__solid"]).sum()))
    assert np.array_equal(nei, g[f"{name}__nei_solid"]), (name, int((nei != g[f"{name}__nei_solid"]).sum()))


def test_stl_vertices_round_trip():
    """The text round trip changes vertices by less than the 7 printed digits."""
    tris = MESHES["ellipsoid_q19"]()
    v = stl_vertices(tris)
    assert v.shape == tris.shape and np.abs(v - tris).max() < 1e-5 * np.abs(tris).max()
