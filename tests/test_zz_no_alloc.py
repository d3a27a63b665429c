"""lbffs_mass_noalloc against lbffs_mass, through the C ABI.

lbffs_mass_noalloc takes float32 populations and solid flags that the caller already holds on
the device and writes the FP64 fluid mass to a caller-owned device double; its per-block partial
sums live in the library's fixed scratch array.  Both entry points add the same per-cell FP32
densities in FP64, in different orders, so they agree to FP64 round-off: the bar is 1e-12
relative.  Two calls in a row, the second on a smaller lattice than the first, show that the
shared scratch carries nothing from one call into the next.
"""
import ctypes as C

import numpy as np
import pytest

from lbffs_gb300 import case as K
from lbffs_gb300.geometry import cylinder_z

pytestmark = pytest.mark.gpu

MAX_CELLS = 268435456  # LBFFS_NOALLOC_MAX_CELLS in include/lbffs_cuda.h
REL_TOL = 1e-12


def _bind(lib):
    fn = lib.lbffs_mass_noalloc
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _lattice_case(L, c, steps):
    lat = L.Lattice(c.nx, c.ny, c.nz, q=c.q, collision="rr", wall="bb")
    lat.load_case(c)
    lat.step(steps, store_fields=0)
    lat.synchronize()
    return lat


def _noalloc_mass(fn, lat, solid, out, slot):
    import torch
    f_d = torch.from_numpy(lat.download("f")).to("cuda:0")
    s_d = torch.from_numpy(np.ascontiguousarray(solid, dtype=np.uint8)).to("cuda:0")
    stream = torch.cuda.current_stream(0)
    rc = fn(0, f_d.data_ptr(), s_d.data_ptr(), lat.q, lat.E, out.data_ptr() + 8 * slot, stream.cuda_stream)
    stream.synchronize()
    return rc


def test_noalloc_mass_matches_lbffs_mass_twice(cuda_lib):
    import torch

    import lbffs_gb300 as L
    fn = _bind(cuda_lib)
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda:0")

    # first call: D3Q27 cavity, 40^3 cells (8 blocks of partials)
    big = K.make_case(40, 40, 40, 27, K.cavity_faces(0.05), nu=0.02)
    lat_big = _lattice_case(L, big, 20)
    assert _noalloc_mass(fn, lat_big, big.solid, out, 0) == 0, cuda_lib.lbffs_last_error(None)
    m_big = lat_big.mass()

    # second call: D3Q19 channel past a cylinder with solid cells, 32x20x6 (a single block)
    solid, sdf = cylinder_z(32, 20, 6, 10.3, 9.8, 3.6)
    small = K.make_case(32, 20, 6, 19, K.channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
    lat_small = _lattice_case(L, small, 30)
    assert _noalloc_mass(fn, lat_small, small.solid, out, 1) == 0, cuda_lib.lbffs_last_error(None)
    m_small = lat_small.mass()

    got = out.cpu().numpy()
    assert abs(got[0] - m_big) <= REL_TOL * abs(m_big), (got[0], m_big)
    assert abs(got[1] - m_small) <= REL_TOL * abs(m_small), (got[1], m_small)
    assert (small.solid != 0).any()


def test_noalloc_mass_rejects_oversize(cuda_lib):
    import torch
    fn = _bind(cuda_lib)
    f_d = torch.zeros(19 * 8, dtype=torch.float32, device="cuda:0")
    s_d = torch.zeros(8, dtype=torch.uint8, device="cuda:0")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda:0")
    rc = fn(0, f_d.data_ptr(), s_d.data_ptr(), 19, MAX_CELLS + 1, out.data_ptr(), None)
    assert rc == -1
    assert b"exceeds the maximum" in cuda_lib.lbffs_last_error(None)
    torch.cuda.synchronize()
    assert out.item() == 7.0  # nothing was launched


def test_noalloc_mass_empty_and_bad_arguments(cuda_lib):
    """n_cells = 0 writes 0.0; q other than 19 / 27 and null pointers are refused with LBFFS_E_ARG and
    leave the output untouched."""
    import torch
    fn = _bind(cuda_lib)
    f_d = torch.ones(27 * 8, dtype=torch.float32, device="cuda:0")
    s_d = torch.zeros(8, dtype=torch.uint8, device="cuda:0")
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream(0)
    assert fn(0, f_d.data_ptr(), s_d.data_ptr(), 19, 0, out.data_ptr(), stream.cuda_stream) == 0
    stream.synchronize()
    assert out.item() == 0.0
    out.fill_(7.0)
    torch.cuda.synchronize()
    assert fn(0, f_d.data_ptr(), s_d.data_ptr(), 20, 8, out.data_ptr(), None) == -1
    assert fn(0, None, s_d.data_ptr(), 19, 8, out.data_ptr(), None) == -1
    assert fn(0, f_d.data_ptr(), s_d.data_ptr(), 19, 8, None, None) == -1
    torch.cuda.synchronize()
    assert out.item() == 7.0
