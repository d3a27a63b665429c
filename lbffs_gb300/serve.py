"""Host mirror of the serving ABI (``lbffs_server_*`` in include/lbffs_cuda.h).

A :class:`Server` keeps many lattice solves resident on one GPU and advances all of them with
batched launches replayed from a CUDA graph; queued solves are admitted as slots and HBM free
up.  Each solve is a :class:`lbffs_gb300.case.Case` plus its step count and selections, and
computes the same numbers as a :class:`lbffs_gb300.Lattice` running it alone.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import COLLISION, SGS, STORAGE, WALL, Desc, LbffsError, StepParams, load_library

QUEUED, RUNNING, DONE, FAILED = 0, 1, 2, -1
RESULT_FIELDS = {"rho": 13, "u": 14, "v": 15, "w": 16, "f": 0}


class ServerDesc(C.Structure):
    _fields_ = [("device", C.c_int), ("hbm_budget", C.c_size_t), ("max_cases", C.c_int),
                ("steps_per_round", C.c_int)]


class CaseDesc(C.Structure):
    _fields_ = [("desc", Desc), ("params", StepParams), ("nsteps", C.c_longlong), ("want_f", C.c_int),
                ("boundary", C.c_void_p), ("boundary1", C.c_void_p), ("boundary2", C.c_void_p),
                ("boundary3", C.c_void_p), ("solid", C.c_void_p), ("nei_solid", C.c_void_p), ("sdf", C.c_void_p),
                ("u0", C.c_void_p), ("v0", C.c_void_p), ("w0", C.c_void_p), ("omega", C.c_void_p),
                ("f", C.c_void_p)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("failed", C.c_longlong),
                ("resident", C.c_longlong), ("queued", C.c_longlong), ("rounds", C.c_longlong),
                ("graph_builds", C.c_longlong), ("cell_updates", C.c_double), ("elapsed_s", C.c_double),
                ("latency_p50_s", C.c_double), ("latency_p99_s", C.c_double), ("latency_mean_s", C.c_double),
                ("latency_max_s", C.c_double), ("queue_wait_p50_s", C.c_double), ("queue_wait_p99_s", C.c_double),
                ("hbm_in_use", C.c_size_t), ("hbm_peak", C.c_size_t), ("hbm_capacity", C.c_size_t),
                ("gpu_busy_s", C.c_double), ("build_s", C.c_double), ("mean_resident", C.c_double)]


def _bind(lib):
    vp, i, ll = C.c_void_p, C.c_int, C.c_longlong
    sig = {
        "lbffs_server_create": ([C.POINTER(ServerDesc), C.POINTER(vp)], i),
        "lbffs_server_destroy": ([vp], i),
        "lbffs_server_submit": ([vp, C.POINTER(CaseDesc), C.POINTER(ll)], i),
        "lbffs_server_poll": ([vp, ll, C.POINTER(i)], i),
        "lbffs_server_wait": ([vp, ll, C.c_double], i),
        "lbffs_server_result": ([vp, ll, i, vp, C.c_size_t], i),
        "lbffs_server_release": ([vp, ll], i),
        "lbffs_server_get_stats": ([vp, C.POINTER(ServerStats)], i),
        "lbffs_server_error": ([vp, ll], C.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Server:
    def __init__(self, hbm_budget=8 << 30, max_cases=64, steps_per_round=16, device=0):
        self.lib = _bind(load_library())
        self.device = int(device)
        d = ServerDesc(self.device, int(hbm_budget), int(max_cases), int(steps_per_round))
        h = C.c_void_p()
        rc = self.lib.lbffs_server_create(C.byref(d), C.byref(h))
        if rc != 0:
            raise LbffsError(rc, self.lib.lbffs_last_error(None).decode())
        self.h = h
        self._shape = {}

    def _check(self, rc, cid=-1):
        if rc != 0:
            raise LbffsError(rc, self.lib.lbffs_server_error(self.h, cid).decode())

    def submit(self, c, nsteps, storage="fp32", wall="bb", les=0.0, dpdx=0.0, omega_b=0.1, spz_width=0.1,
               cs=0.1, want_f=False, from_rest=False):
        """Queue case ``c`` (a :class:`case.Case`) for ``nsteps`` steps; returns its id."""
        keep = [np.ascontiguousarray(getattr(c, k), dtype=np.int32)
                for k in ("boundary", "boundary1", "boundary2", "boundary3")]
        solid = np.ascontiguousarray(c.solid, dtype=np.uint8)
        nei = np.ascontiguousarray(c.nei_solid, dtype=np.uint8)
        fl = {k: np.ascontiguousarray(getattr(c, k), dtype=np.float32) for k in ("sdf", "u0", "v0", "w0", "omega")}
        f = None if from_rest else np.ascontiguousarray(c.f, dtype=np.float32)
        desc = Desc(c.nx, c.ny, c.nz, c.q, STORAGE[storage], COLLISION["rr"], SGS["smag"], WALL[wall], self.device,
                    float(cs))
        params = StepParams(dpdx, 1.0, les, omega_b, spz_width, 0.01, 0)
        cd = CaseDesc(desc, params, int(nsteps), int(bool(want_f)), _ptr(keep[0]), _ptr(keep[1]), _ptr(keep[2]),
                      _ptr(keep[3]), _ptr(solid), _ptr(nei), _ptr(fl["sdf"]), _ptr(fl["u0"]), _ptr(fl["v0"]),
                      _ptr(fl["w0"]), _ptr(fl["omega"]), _ptr(f))
        cid = C.c_longlong()
        self._check(self.lib.lbffs_server_submit(self.h, C.byref(cd), C.byref(cid)))
        self._shape[cid.value] = (c.q, c.nx * c.ny * c.nz)
        return cid.value

    def state(self, cid):
        st = C.c_int()
        self._check(self.lib.lbffs_server_poll(self.h, cid, C.byref(st)), cid)
        return st.value

    def wait(self, cid, timeout=600.0):
        self._check(self.lib.lbffs_server_wait(self.h, cid, float(timeout)), cid)

    def result(self, cid, field="u"):
        q, e = self._shape[cid]
        out = np.empty(q * e if field == "f" else e, np.float32)
        self._check(self.lib.lbffs_server_result(self.h, cid, RESULT_FIELDS[field], _ptr(out), out.nbytes), cid)
        return out

    def release(self, cid):
        self._check(self.lib.lbffs_server_release(self.h, cid), cid)
        self._shape.pop(cid, None)

    def stats(self):
        st = ServerStats()
        self._check(self.lib.lbffs_server_get_stats(self.h, C.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbffs_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
