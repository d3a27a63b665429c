"""Population upload / download through the C ABI: the padded device planes hold exactly what was
uploaded (FP32: pitched copies into the planes; 2-byte storage: the stored value of each element),
for grids whose rows are not a multiple of the 32-byte sector and for both population copies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
@pytest.mark.parametrize("shape", [(37, 11, 7), (64, 3, 5), (1, 1, 1), (130, 9, 2)])
def test_population_upload_download_round_trip(cuda_lib, storage, shape):
    import lbffs_gb300 as L
    from lbffs_gb300 import case as K
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 7 + ny * 3 + nz)
    w = K.lattice(19)[1].astype(np.float64)
    f = (w[:, None] * (1.0 + 0.05 * (rng.random((19, nx * ny * nz)) - 0.5))).astype(np.float32).reshape(-1)
    lat = L.Lattice(nx, ny, nz, storage=storage)
    lat.upload("f", f)
    g = lat.download("f")
    if storage == "fp32":
        assert np.array_equal(g, f)
    else:
        # a second round trip of the stored values is exact
        lat.upload("f", g)
        assert np.array_equal(lat.download("f"), g)
        # |f - w| <= 0.025 w0 = 8.3e-3: FP16S rounds 2^15 (f - w) to an 11-bit significand (half an
        # ulp: 4.1e-6 in f), BF16S rounds f - w to 8 bits (3.3e-5)
        assert np.abs(g - f).max() < (5e-6 if storage == "fp16s" else 4e-5)
    lat.close()
