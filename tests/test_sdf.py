"""LES wall-distance set-up (lbffs_build_sdf) against the reference's host sequence
(ns.cpp:200-225: setSDF per STL patch, then setSDFnearBwalls), on the fixtures the reference
wrote (tests/golden/setup_voxels.npz, ``__sdf``).

The CPU restatement in oracle/sdf.py is pinned bit for bit to those fixtures first; the device
result is then compared with the fixtures directly.  Tolerance: the device forms r^-p in double
by repeated squaring where the reference calls the C library's pow, so in rare cells a float
running sum can round the other way; at most 1e-4 of the cells (and never more than 8) may
differ, each by at most 1e-5 relative (1e-5 absolute near zero).  Every other cell is bit-exact.
"""
import numpy as np
import pytest

from oracle import sdf as S
from test_voxel import MESHES, golden_case, read_mesh

VOXEL_BC = (1, 1, 1, 1, 0, 0)


def face_codes(nx, ny, nz, bc):
    """boundary1..3 as the fixture driver fills them (face cells only, ns.cpp's face flags)."""
    E = nx * ny * nz
    b = [np.zeros(E, np.int32) for _ in range(3)]
    B1, B2, B3 = (x.reshape(nz, ny, nx) for x in b)
    # far face first: the near face wins on a one-cell axis, as the driver's if / else if
    B1[:, :, nx - 1], B2[:, ny - 1, :], B3[nz - 1, :, :] = bc[1], bc[3], bc[5]
    B1[:, :, 0], B2[:, 0, :], B3[0, :, :] = bc[0], bc[2], bc[4]
    return b


def case_bc(g, name):
    key = f"{name}__bc"
    return tuple(int(x) for x in g[key]) if key in g.files else VOXEL_BC


@pytest.mark.parametrize("name", ["ellipsoid_q19", "two_patch_q19"])
def test_oracle_sdf_matches_reference_fixture(name):
    g, q, nx, ny, nz = golden_case(name)
    v, n, counts = read_mesh(name)
    b1, b2, b3 = face_codes(nx, ny, nz, case_bc(g, name))
    sdf = S.les_sdf(v, n, counts, g[f"{name}__nei_solid"], b1, b2, b3, nx, ny, nz)
    ref = g[f"{name}__sdf"]
    assert np.array_equal(sdf, ref), int((sdf != ref).sum())


def test_oracle_last_patch_decides():
    """Each setSDF call rewrites every near cell: two patches give the second patch's field."""
    name = "two_patch_q19"
    g, q, nx, ny, nz = golden_case(name)
    v, n, counts = read_mesh(name)
    b = face_codes(nx, ny, nz, case_bc(g, name))
    nei = g[f"{name}__nei_solid"]
    both = S.les_sdf(v, n, counts, nei, *b, nx, ny, nz)
    last = S.les_sdf(v[counts[0]:], n[counts[0]:], counts[1:], nei, *b, nx, ny, nz)
    assert np.array_equal(both, last)


def check_close(got, ref, what):
    bad = np.flatnonzero(got != ref)
    limit = min(8, max(1, int(1e-4 * ref.size)))
    assert bad.size <= limit, (what, bad.size, bad[:8], got[bad[:8]], ref[bad[:8]])
    if bad.size:
        r = ref[bad].astype(np.float64)
        d = np.abs(got[bad].astype(np.float64) - r)
        assert np.all(d <= 1e-5 * np.maximum(1.0, np.abs(r))), (what, d.max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(MESHES))
def test_build_sdf_matches_reference(cuda_lib, name):
    import lbffs_gb300 as L
    g, q, nx, ny, nz = golden_case(name)
    v, n, counts = read_mesh(name)
    b1, b2, b3 = face_codes(nx, ny, nz, case_bc(g, name))
    lat = L.Lattice(nx, ny, nz, q=q, wall="ibb" if q == 27 else "bb")
    lat.upload("boundary1", b1)
    lat.upload("boundary2", b2)
    lat.upload("boundary3", b3)
    lat.voxelize(v, invert=bool(int(g[f"{name}__invert"][0])))
    lat.build_sdf(v, n, counts)
    sdf = lat.download("sdf")
    # a second call on the same context gives the same field
    lat.build_sdf(v, n, counts)
    again = lat.download("sdf")
    lat.close()
    check_close(sdf, g[f"{name}__sdf"], name)
    assert np.array_equal(sdf, again)


@pytest.mark.gpu
def test_build_sdf_walls_only_and_options(cuda_lib):
    """No STL patch: only sdfIni and the face pass; dr_walls < 0 skips the face pass; other dr."""
    import lbffs_gb300 as L
    name = "two_patch_q19"
    g, q, nx, ny, nz = golden_case(name)
    v, n, counts = read_mesh(name)
    b = face_codes(nx, ny, nz, (1, 1, 0, 1, 1, 1))
    nei = g[f"{name}__nei_solid"]
    lat = L.Lattice(nx, ny, nz, q=q)
    for k, arr in zip(("boundary1", "boundary2", "boundary3"), b):
        lat.upload(k, arr)
    lat.upload("nei_solid", nei)
    lat.build_sdf(v[:0], n[:0], [], dr_walls=2.0)
    assert np.array_equal(lat.download("sdf"), S.les_sdf(v[:0], n[:0], [], nei, *b, nx, ny, nz, dr_walls=2.0))
    lat.build_sdf(v, n, counts, dr=4.0, p=3.5, sdf_ini=-1.0, dr_walls=-1.0)
    got = lat.download("sdf")
    want = S.les_sdf(v, n, counts, nei, *b, nx, ny, nz, dr=4.0, p=3.5, sdf_ini=-1.0, dr_walls=-1.0)
    check_close(got, want, "dr4 p3.5")
    with pytest.raises(L.LbffsError):
        lat.build_sdf(v, n, [counts[0], -1])
    with pytest.raises(L.LbffsError):
        lat.build_sdf(v, n, counts, dr=float("nan"))
    lat.close()
