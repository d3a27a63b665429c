"""GB300 lattice-Boltzmann step for LBFFS.

The product is ``liblbffs_cuda.so`` (C ABI in ``include/lbffs_cuda.h``); this
package is its Python host-side mirror of the reference driver
(``D3Q19_opencl/ns.cpp``): a :class:`Lattice` owns one device context, takes the
reference's host arrays (``case.Case``) and advances them with the CUDA step.

There is no CPU fallback: importing works without a GPU, but creating a
:class:`Lattice` needs the compiled library and a CUDA device and raises
otherwise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import case  # noqa: F401  (re-exported)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbffs_cuda.so")

# enum values of include/lbffs_cuda.h
FP32, FP16S, BF16S = 0, 1, 2
STORAGE = {"fp32": FP32, "fp16s": FP16S, "bf16s": BF16S}
COLLISION = {"rr": 0, "cumulant": 1}
SGS = {"smag": 0, "smagorinsky": 0, "wale": 1}
WALL = {"bb": 0, "ibb": 1}
DAMPING = {"wall": 0, "vandriest": 1, "none": 2}
FIELDS = {"f": 0, "boundary": 1, "boundary1": 2, "boundary2": 3, "boundary3": 4, "sdf": 5, "solid": 6,
          "nei_solid": 7, "u0": 8, "v0": 9, "w0": 10, "omega": 11, "tau_sgs": 12, "rho": 13, "u": 14, "v": 15,
          "w": 16, "fwx": 17, "fwy": 18, "fwz": 19, "gx": 20, "gy": 21, "gz": 22, "out_rho": 23, "out_u": 24,
          "out_v": 25, "out_w": 26, "u_mean": 27, "v_mean": 28, "w_mean": 29}
FIELD_DTYPE = {"boundary": np.int32, "boundary1": np.int32, "boundary2": np.int32, "boundary3": np.int32,
               "solid": np.uint8, "nei_solid": np.uint8}
E_ARG, E_CUDA, E_STATE, E_UNSUPPORTED, E_NONFINITE = -1, -2, -3, -4, -5


class LbffsError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"lbffs error {code}: {msg}")
        self.code = code


class Desc(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("q", C.c_int), ("storage", C.c_int),
                ("collision", C.c_int), ("sgs", C.c_int), ("wall", C.c_int), ("device", C.c_int), ("cs", C.c_float),
                ("damping", C.c_int)]


class StepParams(C.Structure):
    _fields_ = [("dpdx", C.c_float), ("rho_av", C.c_float), ("les", C.c_float), ("omega_b", C.c_float),
                ("spz_width", C.c_float), ("clim", C.c_float), ("store_fields", C.c_int)]


class OutputParams(C.Structure):
    _fields_ = [("dpdx", C.c_float), ("c", C.c_float), ("L", C.c_float), ("out_interval", C.c_int),
                ("force_coeffs", C.c_int)]


class OutputResult(C.Structure):
    _fields_ = [("rho_av", C.c_float), ("rho_max", C.c_float), ("rho_min", C.c_float), ("u_ave", C.c_float),
                ("time_mean", C.c_float), ("n_fluid", C.c_longlong), ("fw", C.c_double * 3),
                ("g_ibm", C.c_double * 3)]


class Motion(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("u_trans", "v_trans", "w_trans", "rot_x", "rot_y", "rot_z", "axis_x",
                                         "axis_y", "axis_z", "rot_omega", "amp_x", "amp_y", "amp_z", "period")]


_lib = None


def library_path():
    return LIB_PATH


def load_library():
    """Load liblbffs_cuda.so; raise if it has not been built (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python lbffs_gb300/build.py`")
    lib = C.CDLL(LIB_PATH)
    vp, i, sz = C.c_void_p, C.c_int, C.c_size_t
    sig = {
        "lbffs_create": ([C.POINTER(Desc), C.POINTER(vp)], i),
        "lbffs_destroy": ([vp], i),
        "lbffs_last_error": ([vp], C.c_char_p),
        "lbffs_upload": ([vp, i, vp, sz], i),
        "lbffs_download": ([vp, i, vp, sz], i),
        "lbffs_step": ([vp, C.POINTER(StepParams), i], i),
        "lbffs_synchronize": ([vp], i),
        "lbffs_force_sum": ([vp, C.POINTER(C.c_double)], i),
        "lbffs_mass": ([vp, C.POINTER(C.c_double)], i),
        "lbffs_links": ([vp, C.POINTER(C.c_longlong), C.POINTER(C.c_uint), C.c_longlong, C.POINTER(C.c_longlong)], i),
        "lbffs_set_markers": ([vp, C.POINTER(C.c_float), i], i),
        "lbffs_get_markers": ([vp, C.POINTER(C.c_float), i], i),
        "lbffs_set_motion": ([vp, C.POINTER(Motion)], i),
        "lbffs_ibm_force_sum": ([vp, C.POINTER(C.c_double)], i),
        "lbffs_get_stream": ([vp, C.POINTER(vp)], i),
        "lbffs_set_timing": ([vp, i], i),
        "lbffs_kernel_time": ([vp, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong)], i),
        "lbffs_cell_counts": ([vp, C.POINTER(C.c_longlong)], i),
        "lbffs_init_rest": ([vp], i),
        "lbffs_set_bulk_kernel": ([vp, i], i),
        "lbffs_set_special_kernel": ([vp, i], i),
        "lbffs_set_border_pulls": ([vp, i], i),
        "lbffs_voxelize": ([vp, C.POINTER(C.c_float), C.c_longlong, i], i),
        "lbffs_output": ([vp, C.POINTER(OutputParams), C.POINTER(OutputResult)], i),
        "lbffs_write_vtk": ([vp, C.c_char_p, i, C.POINTER(OutputParams)], i),
        "lbffs_write_restart": ([vp, C.c_char_p, i], i),
        "lbffs_read_restart": ([vp, C.c_char_p, C.POINTER(C.c_int)], i),
        "lbffs_io_wait": ([vp], i),
        "lbffs_build_sdf": ([vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_longlong), i, C.c_float,
                             C.c_float, C.c_float, C.c_float], i),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class Lattice:
    """One device lattice: the C-ABI context plus host-side conveniences.

    ``q`` 19 or 27; ``storage`` "fp32" | "fp16s" | "bf16s" (BF16S: below the 1e-3 velocity-error bar
    that FP16S meets); ``collision`` "rr" | "cumulant";
    ``sgs`` "smag" | "wale"; ``wall`` "bb" | "ibb"; ``damping`` (near-wall damping of the Smagorinsky
    eddy viscosity) "wall" (the reference's live factor) | "vandriest" | "none".
    """

    def __init__(self, nx, ny, nz, q=19, storage="fp32", collision="rr", sgs="smag", wall="bb", device=0, cs=0.1,
                 damping="wall"):
        self.lib = load_library()
        self.nx, self.ny, self.nz, self.q = int(nx), int(ny), int(nz), int(q)
        self.E = self.nx * self.ny * self.nz
        d = Desc(self.nx, self.ny, self.nz, self.q, STORAGE[storage], COLLISION[collision], SGS[sgs], WALL[wall],
                 int(device), float(cs), DAMPING[damping])
        h = C.c_void_p()
        self._check(self.lib.lbffs_create(C.byref(d), C.byref(h)), None)
        self.h = h
        self.storage = storage

    def _check(self, rc, h="self"):
        if rc != 0:
            hh = self.h if h == "self" else h
            msg = self.lib.lbffs_last_error(hh).decode()
            raise LbffsError(rc, msg)

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbffs_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- fields ----
    def upload(self, name, arr):
        dt = FIELD_DTYPE.get(name, np.float32)
        a = np.ascontiguousarray(arr, dtype=dt)
        self._check(self.lib.lbffs_upload(self.h, FIELDS[name], _ptr(a), a.nbytes))

    def download(self, name):
        dt = FIELD_DTYPE.get(name, np.float32)
        n = self.q * self.E if name == "f" else self.E
        out = np.empty(n, dtype=dt)
        self._check(self.lib.lbffs_download(self.h, FIELDS[name], _ptr(out), out.nbytes))
        return out

    def load_case(self, c):
        """Upload every array of a :class:`case.Case` (the buffers of ns.cpp:405-436)."""
        for name, key in (("boundary", "boundary"), ("boundary1", "boundary1"), ("boundary2", "boundary2"),
                          ("boundary3", "boundary3"), ("u0", "u0"), ("v0", "v0"), ("w0", "w0"), ("solid", "solid"),
                          ("nei_solid", "nei_solid"), ("sdf", "sdf"), ("omega", "omega"), ("f", "f")):
            self.upload(name, getattr(c, key))

    # ---- stepping ----
    def step(self, n=1, dpdx=0.0, les=0.0, omega_b=0.1, spz_width=0.1, clim=0.01, rho_av=1.0, store_fields=1):
        p = StepParams(dpdx, rho_av, les, omega_b, spz_width, clim, int(store_fields))
        self._check(self.lib.lbffs_step(self.h, C.byref(p), int(n)))

    def voxelize(self, vertices, invert=False):
        """setSolid + setNeiSolid of a closed triangle surface on the device (src/walls.hpp).

        ``vertices``: (ntri, 3, 3) float32 in lattice units as the reference holds them after reading
        the STL (stl.hpp normalizeSTLv)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 9)
        self._check(self.lib.lbffs_voxelize(self.h, v.ctypes.data_as(C.POINTER(C.c_float)), v.shape[0],
                                            int(bool(invert))))

    def build_sdf(self, vertices, normals, patch_ntri=None, dr=10.0, p=7.0, sdf_ini=10000.0, dr_walls=3.0):
        """The LES wall-distance field of ns.cpp:200-225 on the device: setSDF per STL patch around
        the current neiSolid, then setSDFnearBwalls on the uploaded boundary1..3 codes.

        ``vertices``: (ntri, 3, 3) float32 as for :meth:`voxelize`; ``normals``: (ntri, 3) facet
        normals as read from the STL; ``patch_ntri``: triangles per patch (default: one patch)."""
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 9)
        n = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 3)
        if n.shape[0] != v.shape[0]:
            raise ValueError("one normal per triangle")
        pn = np.ascontiguousarray([v.shape[0]] if patch_ntri is None else patch_ntri, dtype=np.int64)
        self._check(self.lib.lbffs_build_sdf(self.h, v.ctypes.data_as(C.POINTER(C.c_float)),
                                             n.ctypes.data_as(C.POINTER(C.c_float)),
                                             pn.ctypes.data_as(C.POINTER(C.c_longlong)), int(pn.size), float(dr),
                                             float(p), float(sdf_ini), float(dr_walls)))

    # ---- output step (write.hpp) ----
    def output(self, dpdx=0.0, c=1.0, L=1.0, out_interval=0, force_coeffs=False):
        """rho / u / v / w from the current populations and write.hpp's reductions, on the device;
        returns the scalars as a dict (the fields: ``download("out_rho")`` ...)."""
        p = OutputParams(dpdx, c, L, int(out_interval), int(bool(force_coeffs)))
        r = OutputResult()
        self._check(self.lib.lbffs_output(self.h, C.byref(p), C.byref(r)))
        return {"rho_av": r.rho_av, "rho_max": r.rho_max, "rho_min": r.rho_min, "u_ave": r.u_ave,
                "time_mean": r.time_mean, "n_fluid": r.n_fluid, "fw": list(r.fw), "g_ibm": list(r.g_ibm)}

    def write_vtk(self, path, binary=False, c=1.0, L=1.0, force_coeffs=False):
        """Queue the VTK file of the last :meth:`output`; returns at once (see :meth:`io_wait`)."""
        p = OutputParams(0.0, c, L, 0, int(bool(force_coeffs)))
        self._check(self.lib.lbffs_write_vtk(self.h, os.fsencode(path), int(bool(binary)), C.byref(p)))

    def write_restart(self, path, nt):
        """Queue the restart file (data.dat layout) of the current populations."""
        self._check(self.lib.lbffs_write_restart(self.h, os.fsencode(path), int(nt)))

    def read_restart(self, path):
        nt = C.c_int()
        self._check(self.lib.lbffs_read_restart(self.h, os.fsencode(path), C.byref(nt)))
        return nt.value

    def io_wait(self):
        self._check(self.lib.lbffs_io_wait(self.h))

    def set_bulk_kernel(self, kind):
        """D3Q19 bulk kernel variant: 0 per-thread loads, 1 row-staged bulk copies (same results)."""
        self._check(self.lib.lbffs_set_bulk_kernel(self.h, int(kind)))

    def set_special_kernel(self, kind):
        """Boundary kernel mapping: 0 one thread per listed cell, 1 a lane group per cell, -1 by the
        list's length (same results)."""
        self._check(self.lib.lbffs_set_special_kernel(self.h, int(kind)))

    def set_border_pulls(self, enabled):
        """Face streaming across the grid's border: 1 (default) read where it takes each population
        when the faces allow, 0 a ghost-layer fill before every step (same results)."""
        self._check(self.lib.lbffs_set_border_pulls(self.h, int(enabled)))

    def init_rest(self):
        """Both population copies at rest (f_q = w_q) without a host upload."""
        self._check(self.lib.lbffs_init_rest(self.h))

    def synchronize(self):
        self._check(self.lib.lbffs_synchronize(self.h))

    # ---- reductions and tables ----
    def force_sum(self):
        out = (C.c_double * 3)()
        self._check(self.lib.lbffs_force_sum(self.h, out))
        return np.array(out[:])

    def mass(self):
        out = C.c_double()
        self._check(self.lib.lbffs_mass(self.h, C.byref(out)))
        return out.value

    def links(self):
        n = C.c_longlong()
        self._check(self.lib.lbffs_links(self.h, None, None, 0, C.byref(n)))
        cells = np.empty(max(n.value, 1), np.int64)
        masks = np.empty(max(n.value, 1), np.uint32)
        self._check(self.lib.lbffs_links(self.h, cells.ctypes.data_as(C.POINTER(C.c_longlong)),
                                         masks.ctypes.data_as(C.POINTER(C.c_uint)), n.value, C.byref(n)))
        return cells[:n.value], masks[:n.value]

    def cell_counts(self):
        out = (C.c_longlong * 4)()
        self._check(self.lib.lbffs_cell_counts(self.h, out))
        return dict(zip(("fluid", "special", "link", "store"), out[:]))

    # ---- IBM ----
    def set_markers(self, xyz):
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        self._check(self.lib.lbffs_set_markers(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), a.shape[0]))
        self._n_markers = a.shape[0]

    def markers(self):
        out = np.empty((self._n_markers, 3), np.float32)
        self._check(self.lib.lbffs_get_markers(self.h, out.ctypes.data_as(C.POINTER(C.c_float)), self._n_markers))
        return out

    def set_motion(self, trans=(0, 0, 0), rot=(0, 0, 0), axis=(0, 0, 1), rot_omega=0.0, amp=(0, 0, 0), period=0.0):
        m = Motion(*trans, *rot, *axis, rot_omega, *amp, period)
        self._check(self.lib.lbffs_set_motion(self.h, C.byref(m)))

    def ibm_force_sum(self):
        out = (C.c_double * 3)()
        self._check(self.lib.lbffs_ibm_force_sum(self.h, out))
        return np.array(out[:])

    # ---- timing ----
    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.lbffs_get_stream(self.h, C.byref(s)))
        return s.value

    def set_timing(self, on=True):
        self._check(self.lib.lbffs_set_timing(self.h, int(bool(on))))

    def kernel_time(self, name="bulk"):
        ms, n = C.c_double(), C.c_longlong()
        self._check(self.lib.lbffs_kernel_time(self.h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def macros(self):
        """rho, u, v, w from the current populations as write.hpp's host cal_rhoUVW computes them."""
        cvec, _ = case.lattice(self.q)
        f = self.download("f").reshape(self.q, -1).astype(np.float64)
        rho = f.sum(0)
        return rho, (f * cvec[:, 0:1]).sum(0) / rho, (f * cvec[:, 1:2]).sum(0) / rho, (f * cvec[:, 2:3]).sum(0) / rho
