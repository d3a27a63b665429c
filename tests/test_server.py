"""Serving: continuous batching of many solves on one GPU (lbffs_server_* through ctypes).

Each served case runs the same per-cell code as lbffs_step, so a case's result must be the same
alone in the server, inside a mixed batch (other grid sizes, storage formats, wall models, step
counts, and a case arriving while the batch runs), and through a plain Lattice.  The tolerance
for all three comparisons is exact equality of the float32 fields.
"""
import time

import numpy as np
import pytest

from lbffs_gb300 import case as K
from lbffs_gb300.geometry import cylinder_z

pytestmark = pytest.mark.gpu


def _cavity(n=24, u=0.05, nu=0.02):
    return K.make_case(n, n, n, 19, K.cavity_faces(u), nu=nu)


def _channel(nx=48, ny=24, nz=8):
    solid, sdf = cylinder_z(nx, ny, nz, nx / 4 + 0.3, ny / 2 - 0.2, ny / 7)
    return K.make_case(nx, ny, nz, 19, K.channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)


def _lattice_fields(c, steps, storage, wall):
    import lbffs_gb300 as L
    lat = L.Lattice(c.nx, c.ny, c.nz, q=19, storage=storage, wall=wall)
    lat.load_case(c)
    lat.step(steps, store_fields=1)
    lat.synchronize()
    out = [lat.download(k) for k in ("rho", "u", "v", "w")]
    lat.close()
    return out


def _served_fields(srv, cid):
    return [srv.result(cid, k) for k in ("rho", "u", "v", "w")]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_served_case_equals_alone_and_lattice(cuda_lib):
    from lbffs_gb300.serve import Server
    cav, ch, small = _cavity(), _channel(), _cavity(16, 0.04, 0.03)
    with Server(hbm_budget=1 << 30, max_cases=8, steps_per_round=8) as srv:
        a = srv.submit(cav, 50, "fp32")
        srv.wait(a)
        alone = _served_fields(srv, a)
        ids = {"ch16": srv.submit(ch, 40, "fp16s", wall="ibb"), "cav": srv.submit(cav, 50, "fp32"),
               "small": srv.submit(small, 33, "fp32"), "cav16": srv.submit(cav, 17, "fp16s")}
        time.sleep(0.005)
        ids["late"] = srv.submit(ch, 25, "fp32", wall="bb")  # arrives while the batch runs
        for cid in ids.values():
            srv.wait(cid)
        mix = {k: _served_fields(srv, cid) for k, cid in ids.items()}
        st = srv.stats()
    assert _same(mix["cav"], alone), "cavity differs between alone and in the mix"
    ref = {"cav": _lattice_fields(cav, 50, "fp32", "bb"), "ch16": _lattice_fields(ch, 40, "fp16s", "ibb"),
           "small": _lattice_fields(small, 33, "fp32", "bb"), "cav16": _lattice_fields(cav, 17, "fp16s", "bb"),
           "late": _lattice_fields(ch, 25, "fp32", "bb")}
    for k in ref:
        assert _same(mix[k], ref[k]), f"{k}: served result differs from the Lattice path"
    assert st["completed"] == 6 and st["failed"] == 0
    assert st["latency_p99_s"] >= st["latency_p50_s"] > 0.0
    assert np.abs(alone[1]).max() > 1e-3  # the lid drove a flow


def test_admission_respects_the_hbm_budget(cuda_lib):
    from lbffs_gb300.serve import Server
    cav = _cavity(24)
    budget = 6 << 20  # about one 24^3 FP32 case at a time
    with Server(hbm_budget=budget, max_cases=8, steps_per_round=4) as srv:
        ids = [srv.submit(cav, 12 + 3 * k, "fp32") for k in range(4)]
        for cid in ids:
            srv.wait(cid)
        st = srv.stats()
        res = [_served_fields(srv, cid) for cid in ids]
    assert st["completed"] == 4
    assert 0 < st["hbm_peak"] <= budget
    for k, r in enumerate(res):
        assert _same(r, _lattice_fields(cav, 12 + 3 * k, "fp32", "bb"))


def test_submit_rejects_unsupported_and_oversize(cuda_lib):
    import lbffs_gb300 as L
    from lbffs_gb300.serve import CaseDesc, Server
    cav = _cavity(16)
    with Server(hbm_budget=4 << 20, max_cases=2, steps_per_round=4) as srv:
        with pytest.raises(L.LbffsError) as e:
            srv.submit(_cavity(64), 10, "fp32")  # never fits 4 MiB
        assert e.value.code == L.E_ARG
        cd = CaseDesc()
        cd.desc = L.Desc(16, 16, 16, 27, 0, 0, 0, 0, 0, 0.1)  # D3Q27 is not served
        cd.nsteps = 5
        import ctypes as C
        cid = C.c_longlong()
        assert srv.lib.lbffs_server_submit(srv.h, C.byref(cd), C.byref(cid)) == L.E_UNSUPPORTED
        ok = srv.submit(cav, 5, "fp32")
        srv.wait(ok)
        assert srv.state(ok) == 2


def test_serving_workload_sample_matches_plain_lattices(cuda_lib):
    """Requests drawn like the serving workload (cavity / channel, FP32 / FP16S, started from
    rest), a dozen resident at once: every served field equals the plain Lattice run."""
    import lbffs_gb300 as L
    from lbffs_gb300.serve import Server
    rng = np.random.default_rng(5)
    cases = []
    for k in range(12):
        n = int(rng.integers(12, 40))
        storage = "fp32" if k % 2 == 0 else "fp16s"
        steps = int(rng.integers(5, 40))
        if k % 3 == 2:
            nx, ny, nz = 2 * n, n, max(4, n // 4)
            solid, sdf = cylinder_z(nx, ny, nz, nx / 4.0, ny / 2.0 + 0.2, n / 10.0)
            c = K.make_case(nx, ny, nz, 19, K.channel_faces(0.05), nu=0.02, solid=solid, sdf=sdf)
            wall = "ibb"
        else:
            c = K.make_case(n, n, n, 19, K.cavity_faces(0.05), nu=0.05 * n / 200.0)
            wall = "bb"
        cases.append((c, storage, steps, wall))
    with Server(hbm_budget=1 << 30, max_cases=16, steps_per_round=8) as srv:
        ids = [srv.submit(c, steps, storage=st, wall=wall, from_rest=True) for c, st, steps, wall in cases]
        for cid in ids:
            srv.wait(cid)
        served = [_served_fields(srv, cid) for cid in ids]
    bad = []
    for k, (c, st, steps, wall) in enumerate(cases):
        lat = L.Lattice(c.nx, c.ny, c.nz, storage=st, wall=wall)
        for name in ("boundary", "boundary1", "boundary2", "boundary3", "u0", "v0", "w0", "solid", "nei_solid", "sdf",
                     "omega"):
            lat.upload(name, getattr(c, name))
        lat.init_rest()
        lat.step(steps, store_fields=1)
        lat.synchronize()
        ref = [lat.download(f) for f in ("rho", "u", "v", "w")]
        lat.close()
        if not _same(served[k], ref):
            d = max(float(np.abs(a - b).max()) for a, b in zip(served[k], ref))
            bad.append((k, c.nx, c.ny, c.nz, st, steps, wall, d))
    assert not bad, bad


def test_wide_rows_run_in_row_tiles_and_equal_lattice(cuda_lib):
    """Cases whose rows fill most of a 256-cell row tile (nx >= 180) run in the single-lattice kernel's
    row tiles inside the batch, next to narrow cases in the segment mapping: every served field
    equals the plain Lattice run."""
    from lbffs_gb300.serve import Server
    wide_ch = _channel(192, 24, 6)
    wide_cav = K.make_case(200, 12, 10, 19, K.cavity_faces(0.05), nu=0.03)
    two_tiles = _channel(300, 16, 4)
    runs = [(wide_ch, 30, "fp32", "ibb"), (wide_ch, 23, "fp16s", "ibb"), (wide_cav, 27, "fp32", "bb"),
            (wide_cav, 31, "fp16s", "bb"), (two_tiles, 19, "fp16s", "ibb"), (_cavity(20, 0.05, 0.02), 25, "fp32", "bb")]
    with Server(hbm_budget=1 << 30, max_cases=8, steps_per_round=8) as srv:
        ids = [srv.submit(c, n, st, wall=w) for c, n, st, w in runs]
        for cid in ids:
            srv.wait(cid)
        served = [_served_fields(srv, cid) for cid in ids]
    for k, (c, n, st, w) in enumerate(runs):
        assert _same(served[k], _lattice_fields(c, n, st, w)), (k, c.nx, st)


def test_slot_reuse_under_continuous_admission(cuda_lib):
    """Two slots and one step per round, so every round retires a case and admits the next into
    the slot just freed while the batch of the other slot runs: each served result equals the
    plain Lattice run of the same case and step count (a reused slot's step counter starts at 0)."""
    import lbffs_gb300 as L
    from lbffs_gb300.serve import Server
    rng = np.random.default_rng(11)
    base = [_cavity(12, 0.05, 0.02), _cavity(14, 0.04, 0.03)]
    runs = [(int(rng.integers(0, 2)), int(rng.integers(2, 14)), "fp32" if k % 3 else "fp16s") for k in range(24)]
    with Server(hbm_budget=1 << 28, max_cases=2, steps_per_round=1) as srv:
        ids = []
        for b, steps, st in runs:
            ids.append(srv.submit(base[b], steps, storage=st))
            time.sleep(float(rng.uniform(0.0, 0.002)))
        for cid in ids:
            srv.wait(cid)
        served = [_served_fields(srv, cid) for cid in ids]
    want = {}
    for b, steps, st in runs:
        if (b, steps, st) not in want:
            want[(b, steps, st)] = _lattice_fields(base[b], steps, st, "bb")
    bad = [k for k, r in enumerate(runs) if not _same(served[k], want[r])]
    assert not bad, bad
