"""Population transfers from and to page-locked host memory (one conversion kernel over the host link)
give the same bits as transfers from and to pageable memory (copies through a device staging area).

Both directions, every storage format, both lattices, rows that are not a multiple of 16 bytes long;
and a step after a page-locked upload equals the step after a pageable one (the upload fills both
population copies)."""
import ctypes as C

import numpy as np
import pytest

from lbffs_gb300 import case as K

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("q", [19, 27])
@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
def test_pinned_and_pageable_population_transfers_agree(cuda_lib, storage, q):
    torch = pytest.importorskip("torch")
    import lbffs_gb300 as L
    c = K.make_case(37, 11, 6, q, K.cavity_faces(0.05), nu=0.03)
    rng = np.random.default_rng(q + len(storage))
    f = (c.f + 1e-3 * rng.standard_normal(c.f.shape)).astype(np.float32)
    c.f = f

    def run(pinned):
        lat = L.Lattice(c.nx, c.ny, c.nz, q=q, storage=storage)
        lat.load_case(c)
        if pinned:
            hp = torch.from_numpy(f).pin_memory()
            assert lat.lib.lbffs_upload(lat.h, 0, C.c_void_p(hp.data_ptr()), hp.numel() * 4) == 0
        back = lat.download("f")
        out = torch.empty(f.size, dtype=torch.float32).pin_memory()
        assert lat.lib.lbffs_download(lat.h, 0, C.c_void_p(out.data_ptr()), out.numel() * 4) == 0
        lat.step(3)
        stepped = lat.download("f")
        lat.close()
        return back, out.numpy().copy(), stepped

    a_back, a_pinned_down, a_step = run(False)
    b_back, b_pinned_down, b_step = run(True)
    assert np.array_equal(a_back, b_back)            # pinned upload == pageable upload
    assert np.array_equal(a_pinned_down, a_back)     # pinned download == pageable download
    assert np.array_equal(b_pinned_down, b_back)
    assert np.array_equal(a_step, b_step)            # both copies filled alike
    if storage == "fp32":
        assert np.array_equal(a_back, f)
