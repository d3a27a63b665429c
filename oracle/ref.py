"""ctypes front-end of ``oracle/_ref`` (the reference kernels compiled as C).

Test infrastructure only.  ``RefSolver`` owns numpy copies of every buffer of
``D3Q19_opencl/ns.cpp:405-436`` and advances them with the reference's own
``k_streamingCollision`` (+ IBM kernels) through ``ref_driver.c``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

_FIELDS = ["f", "fTmp", "boundary", "boundary1", "boundary2", "boundary3", "sdf", "solid", "neiSolid", "u0", "v0",
           "w0", "Fwx", "Fwy", "Fwz", "tauSGS", "rho", "u", "v", "w", "omega", "Gx", "Gy", "Gz", "rhoPrev", "uPrev",
           "vPrev", "wPrev"]
_INT = {"boundary", "boundary1", "boundary2", "boundary3"}
_U8 = {"solid", "neiSolid"}


def lib_path(q, sgs="smag", wall="bb", real="f32"):
    if q == 27:
        wall = "ibb"
    return os.path.join(REF_DIR, f"libref_d3q{q}_{sgs}_{wall}_{real}.so")


def available(q=19, sgs="smag", wall="bb", real="f32"):
    return os.path.exists(lib_path(q, sgs, wall, real))


class RefSolver:
    """Runs the reference step on a :class:`lbffs_gb300.case.Case`-like object."""

    def _load(self, case, sgs, wall, real):
        if case.q == 27 and wall != "ibb":
            raise ValueError("the D3Q27 reference always uses interpolated bounce-back (wall='ibb')")
        path = lib_path(case.q, sgs, wall, real)
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        return C.CDLL(path)

    def __init__(self, case, sgs="smag", wall="bb", real="f32", nthreads=0, collision="cumulant", cs=0.1,
                 damping="wall"):
        if damping != "wall" and type(self) is RefSolver:
            raise ValueError("the reference kernels apply only the live near-wall damping (damping='wall')")
        self.lib = self._load(case, sgs, wall, real)
        self.sgs, self.wall, self.collision, self.cs, self.damping = sgs, wall, collision, cs, damping
        self.real = np.float32 if real == "f32" else np.float64
        rt = C.c_float if real == "f32" else C.c_double
        self.rt = rt

        class Fields(C.Structure):
            _fields_ = [(n, C.POINTER(C.c_int) if n in _INT else C.POINTER(C.c_ubyte) if n in _U8 else C.POINTER(rt))
                        for n in _FIELDS]

        class Params(C.Structure):
            _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("dpdx", rt), ("rho_av", rt), ("LES", rt),
                        ("isReadMovingWalls", C.c_int), ("omegaB", rt), ("spzWidth", rt), ("clim", rt),
                        ("nthreads", C.c_int)]

        class Ibm(C.Structure):
            _fields_ = [("markers", C.POINTER(rt)), ("Gmx", C.POINTER(rt)), ("Gmy", C.POINTER(rt)),
                        ("Gmz", C.POINTER(rt)), ("n", C.c_int)] + \
                       [(n, rt) for n in ("uT", "vT", "wT", "rotX", "rotY", "rotZ", "axX", "axY", "axZ", "rotOmega")]

        self._Fields, self._Params, self._Ibm = Fields, Params, Ibm
        self._bind()
        self.case = case
        self.nx, self.ny, self.nz, self.q = case.nx, case.ny, case.nz, case.q
        E = case.elements
        R = self.real
        self.a = {
            "f": case.f.astype(R).copy(), "fTmp": case.f.astype(R).copy(),
            "boundary": case.boundary.astype(np.int32).copy(), "boundary1": case.boundary1.astype(np.int32).copy(),
            "boundary2": case.boundary2.astype(np.int32).copy(), "boundary3": case.boundary3.astype(np.int32).copy(),
            "sdf": case.sdf.astype(R).copy(), "solid": case.solid.astype(np.uint8).copy(),
            "neiSolid": case.nei_solid.astype(np.uint8).copy(), "u0": case.u0.astype(R).copy(),
            "v0": case.v0.astype(R).copy(), "w0": case.w0.astype(R).copy(), "omega": case.omega.astype(R).copy(),
        }
        for n in ("Fwx", "Fwy", "Fwz", "tauSGS", "rho", "u", "v", "w", "Gx", "Gy", "Gz", "rhoPrev", "uPrev", "vPrev",
                  "wPrev"):
            self.a[n] = np.zeros(E, R)
        self.flip = False  # True when the newest populations are in a["fTmp"]
        self.nthreads = nthreads
        self.ibm = None

    def set_ibm(self, markers, uT=0.0, vT=0.0, wT=0.0, rot=(0.0, 0.0, 0.0), axis=(0.0, 0.0, 1.0), rot_omega=0.0):
        m = np.ascontiguousarray(markers, dtype=self.real).ravel().copy()
        n = m.size // 3
        self.ibm_arrays = {"markers": m, "Gmx": np.zeros(n, self.real), "Gmy": np.zeros(n, self.real),
                           "Gmz": np.zeros(n, self.real)}
        self.ibm = (n, uT, vT, wT, rot, axis, rot_omega)

    def _bind(self):
        self.lib.ref_step.argtypes = [C.POINTER(self._Fields), C.POINTER(self._Params), C.POINTER(self._Ibm),
                                      C.c_int]

    def _call(self, F, P, ibm_p, n):
        return self.lib.ref_step(C.byref(F), C.byref(P), ibm_p, n)

    def _ptr(self, arr):
        return arr.ctypes.data_as(C.c_void_p)

    def step(self, n=1, dpdx=0.0, LES=0.0, omegaB=0.1, spzWidth=0.1, clim=0.01, rho_av=1.0, is_read_moving=0):
        F = self._Fields()
        order = dict(self.a)
        if self.flip:
            order["f"], order["fTmp"] = self.a["fTmp"], self.a["f"]
        for name in _FIELDS:
            arr = order[name]
            setattr(F, name, C.cast(self._ptr(arr), dict(self._Fields._fields_)[name]))
        P = self._Params(self.nx, self.ny, self.nz, dpdx, rho_av, LES, is_read_moving, omegaB, spzWidth, clim,
                         self.nthreads)
        ibm_p = None
        if self.ibm is not None:
            n_markers, uT, vT, wT, rot, axis, rot_omega = self.ibm
            I = self._Ibm()
            for key in ("markers", "Gmx", "Gmy", "Gmz"):
                setattr(I, key, C.cast(self._ptr(self.ibm_arrays[key]), C.POINTER(self.rt)))
            I.n = n_markers
            I.uT, I.vT, I.wT = uT, vT, wT
            I.rotX, I.rotY, I.rotZ = rot
            I.axX, I.axY, I.axZ = axis
            I.rotOmega = rot_omega
            ibm_p = C.byref(I)
        rc = self._call(F, P, ibm_p, int(n))
        if rc != 0:
            raise RuntimeError(f"step failed with status {rc}")
        if n % 2 == 1:
            self.flip = not self.flip

    @property
    def f(self):
        return self.a["fTmp"] if self.flip else self.a["f"]

    def field(self, name):
        return self.a[name]

    def macros(self):
        """rho, u, v, w from the newest populations as write.hpp's host cal_rhoUVW does (with dpdx = 0)."""
        c, _ = __import__("lbffs_gb300.case", fromlist=["lattice"]).lattice(self.q)
        f = self.f.reshape(self.q, -1).astype(np.float64)
        rho = f.sum(0)
        return rho, (f * c[:, 0:1]).sum(0) / rho, (f * c[:, 1:2]).sum(0) / rho, (f * c[:, 2:3]).sum(0) / rho


ORACLE_DIR = HERE
SGS = {"smag": 0, "wale": 1}
WALL = {"bb": 0, "ibb": 1}
COLLISION = {"rr": 0, "cumulant": 1}
DAMPING = {"wall": 0, "vandriest": 1, "none": 2}


def oracle_available(real="f32"):
    return os.path.exists(os.path.join(ORACLE_DIR, f"liboracle_{real}.so"))


class OracleSolver(RefSolver):
    """Same interface as :class:`RefSolver`, driven by the CPU restatement ``lbm_oracle.c``.

    ``collision`` selects the D3Q27 operator ("cumulant" as the reference runs, or "rr");
    D3Q19 always uses the recursive-regularised operator.  ``damping`` selects the near-wall
    damping of the Smagorinsky eddy viscosity: "wall" (the reference's live min(1, kappa y / Cs)^2),
    "vandriest" (the reference's commented Van Driest block) or "none".  IBM motion may add a
    sinusoidal displacement (``set_motion``).
    """

    def _load(self, case, sgs, wall, real):
        path = os.path.join(ORACLE_DIR, f"liboracle_{real}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        return C.CDLL(path)

    def _bind(self):
        rt = self.rt

        class Config(C.Structure):
            _fields_ = [("q", C.c_int), ("sgs", C.c_int), ("wall", C.c_int), ("collision", C.c_int), ("cs", rt),
                        ("damping", C.c_int)]

        class Motion(C.Structure):
            _fields_ = [("ampX", rt), ("ampY", rt), ("ampZ", rt), ("period", rt), ("step", C.c_long)]

        self._Config, self._Motion = Config, Motion
        self.cfg = Config(self.q if hasattr(self, "q") else 0, SGS[self.sgs], WALL[self.wall],
                          COLLISION[self.collision], self.cs, DAMPING[self.damping])
        self.motion = Motion(0, 0, 0, 0, 0)
        self.lib.oracle_step_motion.argtypes = [C.POINTER(Config), C.POINTER(self._Fields), C.POINTER(self._Params),
                                                C.POINTER(self._Ibm), C.POINTER(Motion), C.c_int]

    def set_motion(self, amp=(0.0, 0.0, 0.0), period=0.0, step=0):
        self.motion = self._Motion(amp[0], amp[1], amp[2], period, step)

    def _call(self, F, P, ibm_p, n):
        self.cfg.q = self.q
        return self.lib.oracle_step_motion(C.byref(self.cfg), C.byref(F), C.byref(P), ibm_p, C.byref(self.motion), n)


def collide(q, ft, rho, u, v, w, tau, tau_sgs=0.0, omega_b=0.1, dpdx=0.0, clim=0.01, collision="rr", real="f64"):
    """One collision of one cell through the oracle's operator (``oracle_collide``): the populations
    after collision for pre-collision populations ft (u including the half-force shift)."""
    lib = C.CDLL(os.path.join(ORACLE_DIR, f"liboracle_{real}.so"))
    rt = C.c_float if real == "f32" else C.c_double
    dt = np.float32 if real == "f32" else np.float64
    lib.oracle_collide.argtypes = [C.c_int, C.c_int, C.c_void_p] + [rt] * 9 + [C.c_void_p]
    src = np.ascontiguousarray(ft, dtype=dt)
    out = np.zeros(q, dt)
    rc = lib.oracle_collide(q, COLLISION[collision], src.ctypes.data_as(C.c_void_p), rho, u, v, w, tau, tau_sgs,
                            omega_b, dpdx, clim, out.ctypes.data_as(C.c_void_p))
    if rc != 0:
        raise ValueError("oracle_collide: unsupported lattice / operator")
    return out
