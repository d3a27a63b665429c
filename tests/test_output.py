"""Output step (lbffs_output, lbffs_write_vtk, lbffs_write_restart, lbffs_read_restart) against
the reference's own write.hpp, run on the CPU on seeded arrays (tests/golden/output_step.npz,
made by tests/golden/make_golden_output.py through oracle/_ref/output_ref19 / output_ref27).

Tolerances: rho / u / v / w, the time means, rhoMax / rhoMin, uAve, timeMean, the VTK files and
data.dat are compared bit for bit; rho_av within one float ulp (the reference sums rho - 1 in
double sequentially, the device in another order); the FP64 force sums within 1e-12 relative of a
float64 sum (the reference sums in float, so its printed coefficients agree to its own rounding
only).
"""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "output_step.npz")
CASES = ["q19_ascii", "q19_binary", "q27_ascii"]


def fixture():
    return np.load(GOLDEN)


def seq_uave(u, nx, ny, nz, c):
    """write.hpp:51-60: uAve += u * c over the x = 0 plane, j outer, k inner, in float."""
    s = np.float32(0.0)
    c = np.float32(c)
    for j in range(ny):
        for k in range(nz):
            s = np.float32(s + np.float32(u[(k * ny + j) * nx] * c))
    return np.float32(s / np.float32(ny * nz))


@pytest.mark.parametrize("name", CASES)
def test_fixture_console_and_restart_layout(name):
    """write.hpp's console uAve / rhoMax lines agree with the restatements the GPU test uses, and
    data.dat is (nt, nx, ny, nz) followed by the populations."""
    g = fixture()
    for k in (1, 2):
        pre = f"{name}__{k}__"
        q, nx, ny, nz, step = (int(x) for x in g[pre + "spec"][:5])
        c = float(g[pre + "fspec"][1])
        console = g[pre + "console"].tobytes().decode().splitlines()
        assert console[0] == "uAve: %g" % seq_uave(g[pre + "u"], nx, ny, nz, c)
        rho = g[pre + "rho"]
        assert console[1].startswith("rhoMax: %g, rhoMin: %g" % (rho.max(), rho.min()))
        data = g[pre + "data"].tobytes()
        assert np.array_equal(np.frombuffer(data[:16], dtype=np.int32), [step, nx, ny, nz])
        assert np.array_equal(np.frombuffer(data[16:], dtype=np.float32), g[pre + "in_f"])


def _upload_inputs(lat, g, pre, fc):
    lat.upload("f", g[pre + "in_f"])
    lat.upload("tau_sgs", g[pre + "in_tauSGS"])
    for dev, ref in (("omega", "omega"), ("boundary1", "boundary1"), ("boundary2", "boundary2"),
                     ("boundary3", "boundary3"), ("sdf", "sdf"), ("solid", "solid"), ("nei_solid", "neiSolid")):
        lat.upload(dev, g[pre + "in_" + ref])
    if fc:
        for dev, ref in (("fwx", "Fwx"), ("fwy", "Fwy"), ("fwz", "Fwz"), ("gx", "GxIBM"), ("gy", "GyIBM"),
                         ("gz", "GzIBM")):
            lat.upload(dev, g[pre + "in_" + ref])


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_output_step_matches_reference(cuda_lib, name, tmp_path):
    import lbffs_gb300 as L
    g = fixture()
    q, nx, ny, nz = (int(x) for x in g[f"{name}__1__spec"][:4])
    lat = L.Lattice(nx, ny, nz, q=q, wall="ibb" if q == 27 else "bb")
    for k in (1, 2):
        pre = f"{name}__{k}__"
        _, _, _, _, step, fc, binary, interval = (int(x) for x in g[pre + "spec"])
        dpdx, c, Lc, _, _ = (float(x) for x in g[pre + "fspec"])
        _upload_inputs(lat, g, pre, fc)
        r = lat.output(dpdx=dpdx, c=c, L=Lc, out_interval=interval, force_coeffs=bool(fc))
        for dev, ref in (("out_rho", "rho"), ("out_u", "u"), ("out_v", "v"), ("out_w", "w"), ("u_mean", "uMean"),
                         ("v_mean", "vMean"), ("w_mean", "wMean")):
            got = lat.download(dev)
            assert np.array_equal(got, g[pre + ref]), (name, k, dev, int((got != g[pre + ref]).sum()))
        rho = g[pre + "rho"]
        assert np.float32(r["rho_max"]) == rho.max() and np.float32(r["rho_min"]) == rho.min()
        assert np.float32(r["time_mean"]) == g[pre + "time_mean"][0]
        assert np.float32(r["u_ave"]) == seq_uave(g[pre + "u"], nx, ny, nz, c)
        ref_av = g[pre + "rho_av"][0]
        assert abs(np.float32(r["rho_av"]) - ref_av) <= np.spacing(ref_av), (r["rho_av"], ref_av)
        fluid = g[pre + "in_solid"] == 0
        assert r["n_fluid"] == int(fluid.sum())
        if fc:
            for a, key in enumerate(("Fwx", "Fwy", "Fwz")):
                want = g[pre + "in_" + key][fluid].astype(np.float64).sum()
                assert abs(r["fw"][a] - want) <= 1e-12 * max(1.0, abs(want))
            for a, key in enumerate(("GxIBM", "GyIBM", "GzIBM")):
                want = g[pre + "in_" + key][fluid].astype(np.float64).sum()
                assert abs(r["g_ibm"][a] - want) <= 1e-12 * max(1.0, abs(want))
        vtk = tmp_path / f"res{step:08d}.vtk"
        lat.write_vtk(str(vtk), binary=bool(binary), c=c, L=Lc, force_coeffs=bool(fc))
        data = tmp_path / "data.dat"
        lat.write_restart(str(data), step)  # waits for the VTK writer first
        lat.io_wait()
        got = np.frombuffer(vtk.read_bytes(), dtype=np.uint8)
        want = g[pre + "vtk"]
        if not np.array_equal(got, want):
            n = min(got.size, want.size)
            diff = np.flatnonzero(got[:n] != want[:n])
            first = int(diff[0]) if diff.size else n
            pytest.fail(f"{name} output {k}: VTK differs at byte {first} (sizes {got.size} / {want.size}): "
                        f"{bytes(got[max(0, first - 40):first + 40])!r} vs {bytes(want[max(0, first - 40):first + 40])!r}")
        assert data.read_bytes() == g[pre + "data"].tobytes()
    # restart.hpp: the second output's data.dat back into the populations
    ref_data = tmp_path / "ref.dat"
    ref_data.write_bytes(g[f"{name}__2__data"].tobytes())
    lat.upload("f", np.zeros(q * nx * ny * nz, np.float32))
    assert lat.read_restart(str(ref_data)) == int(g[f"{name}__2__spec"][4])
    assert np.array_equal(lat.download("f"), g[f"{name}__2__in_f"])
    lat.close()


@pytest.mark.gpu
def test_output_errors_and_async_overlap(cuda_lib, tmp_path):
    """Writes need an output first; a bad path surfaces at io_wait; a restart of another grid is
    refused; steps may run while a file is being written, and the file holds the state of the call."""
    import lbffs_gb300 as L
    from lbffs_gb300 import case as K
    c = K.make_case(24, 20, 16, 19, K.cavity_faces(0.05), nu=0.02)
    lat = L.Lattice(c.nx, c.ny, c.nz)
    lat.load_case(c)
    with pytest.raises(L.LbffsError):
        lat.write_vtk(str(tmp_path / "a.vtk"))
    lat.step(5)
    lat.output(out_interval=5)
    lat.write_vtk(str(tmp_path / "missing_dir" / "a.vtk"))
    with pytest.raises(L.LbffsError):
        lat.io_wait()
    f5 = lat.download("f")
    lat.write_restart(str(tmp_path / "d5.dat"), 5)
    lat.step(20)  # overlaps the writer; the device copy keeps step 5
    lat.io_wait()
    raw = (tmp_path / "d5.dat").read_bytes()
    assert np.array_equal(np.frombuffer(raw[16:], dtype=np.float32), f5)
    other = L.Lattice(8, 8, 8)
    with pytest.raises(L.LbffsError):
        other.read_restart(str(tmp_path / "d5.dat"))
    other.close()
    lat.close()
