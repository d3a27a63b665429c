"""The two D3Q19 bulk kernels (per-thread loads; row-staged bulk async copies) compute the same
step: populations and macroscopic fields must agree bit for bit after N steps, on the reference
cases and on grids whose rows span several tiles, end in a partial tile, or are not a multiple of
16 bytes long."""
import numpy as np
import pytest

from lbffs_gb300 import case as K
from lbffs_gb300.geometry import cylinder_z
from parity_cases import build

pytestmark = pytest.mark.gpu


def _run(c, run, storage, kind, steps=None):
    import lbffs_gb300 as L
    lat = L.Lattice(c.nx, c.ny, c.nz, q=19, storage=storage, collision=run["collision"], sgs=run["sgs"],
                    wall=run["wall"])
    lat.set_bulk_kernel(kind)
    lat.load_case(c)
    kw = run["kw"]
    lat.step(steps or run["steps"], dpdx=kw.get("dpdx", 0.0), les=kw.get("LES", 0.0),
             spz_width=kw.get("spzWidth", 0.1), store_fields=1)
    lat.synchronize()
    out = {k: lat.download(k) for k in ("f", "rho", "u", "v", "w")}
    lat.close()
    return out


@pytest.mark.parametrize("name", ["cavity_q19", "cavity_q19_les", "cavity_q19_wale", "cylinder_q19_ibb_les_sponge",
                                  "cylinder2d_q19_ibb", "mixed_q19", "density_q19_dpdx", "step_q19_les"])
def test_staged_bulk_equals_per_thread_bulk(cuda_lib, name):
    c, run = build(name)
    a = _run(c, run, "fp32", 0)
    b = _run(c, run, "fp32", 1)
    for k in a:
        assert np.array_equal(a[k], b[k]), (name, k)


@pytest.mark.parametrize("storage", ["fp32", "fp16s", "bf16s"])
@pytest.mark.parametrize("shape", [(300, 20, 6), (130, 9, 5), (257, 12, 4), (37, 11, 7)])
def test_staged_bulk_tiles_and_tails(cuda_lib, storage, shape):
    nx, ny, nz = shape
    solid, sdf = cylinder_z(nx, ny, nz, nx / 3.0, ny / 2.0, min(ny, nx) / 5.0)
    c = K.make_case(nx, ny, nz, 19, K.channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
    run = dict(collision="rr", sgs="smag", wall="ibb", kw={}, steps=25)
    a = _run(c, run, storage, 0)
    b = _run(c, run, storage, 1)
    for k in a:
        assert np.array_equal(a[k], b[k]), (shape, storage, k)
