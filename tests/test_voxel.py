"""Device voxelisation (lbffs_voxelize) against the reference's own host voxeliser: solid and
neiSolid bit for bit on the fixtures the reference wrote (src/walls.hpp setSolid / setNeiSolid run
on seeded ellipsoid meshes, including an inverted fluid/solid case, a 6240-triangle mesh and a
two-patch STL)."""
import os
import tempfile

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
    "two_patch_q19": lambda: [("front", G.ellipsoid_mesh(41, 12, 24, (11.2, 13.7, 12.9), (6.0, 5.0, 5.5))),
                              ("back", G.ellipsoid_mesh(43, 12, 24, (24.6, 14.1, 13.3), (5.5, 6.5, 5.0)))],
}


def read_mesh(name):
    """(vertices, normals, triangles per patch) as the reference reads the fixture's STL text."""
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "walls.stl")
        G.write_ascii_stl(path, MESHES[name]())
        return G.read_ascii_stl(path)


def golden_case(name):
    g = np.load(os.path.join(GOLDEN, "setup_voxels.npz"))
    q, nx, ny, nz = (int(v) for v in g[f"{name}__shape"])
    return g, q, nx, ny, nz


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MESHES))
def test_voxelize_matches_reference_voxeliser(cuda_lib, name):
    import lbffs_gb300 as L
    g, q, nx, ny, nz = golden_case(name)
    invert = bool(int(g[f"{name}__invert"][0]))
    v, _, _ = read_mesh(name)
    lat = L.Lattice(nx, ny, nz, q=q, wall="ibb" if q == 27 else "bb")
    lat.voxelize(v, invert=invert)
    solid = lat.download("solid")
    nei = lat.download("nei_solid")
    lat.close()
    assert np.array_equal(solid, g[f"{name}__solid"]), (name, int((solid != g[f"{name}__solid"]).sum()))
    assert np.array_equal(nei, g[f"{name}__nei_solid"]), (name, int((nei != g[f"{name}__nei_solid"]).sum()))


def test_stl_reader_round_trip():
    """The STL text round trip changes vertices by less than the 7 printed digits; patches and
    normals come back as written."""
    tris = MESHES["ellipsoid_q19"]()
    v, n, counts = read_mesh("ellipsoid_q19")
    assert counts == [len(tris)]
    assert v.shape == tris.shape and np.abs(v - tris).max() < 1e-5 * np.abs(tris).max()
    assert np.abs(np.linalg.norm(n.astype(np.float64), axis=1) - 1.0).max() < 1e-6
    direct = np.array([[[np.float32(f"{x:.6e}") for x in p] for p in t] for t in tris], dtype=np.float32)
    assert np.array_equal(v, direct)
    v2, n2, counts2 = read_mesh("two_patch_q19")
    parts = MESHES["two_patch_q19"]()
    assert counts2 == [len(parts[0][1]), len(parts[1][1])] and v2.shape[0] == n2.shape[0] == sum(counts2)
