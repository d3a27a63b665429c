"""Host-side case setup mirroring LBFFS's driver (``D3Q19_opencl/ns.cpp``).

This module builds the per-cell arrays the reference driver hands to the
device (``ns.cpp:77-377``) so that a case can be set up without the
reference's own C++ host code:

* face boundary codes and wall velocities (``src/setBoundaryConditions.hpp``
  and the ``boundary=1`` face flag of ``ns.cpp:164-177``),
* the equilibrium initialisation (``initialization.hpp``),
* the neighbour-solid predicate (``src/walls.hpp:187-216``),
* the lattice-unit conversions of ``ns.cpp:104-131``.

Boundary-condition codes follow ``src/input.hpp:221-256``.
All arrays are numpy, in the reference's cell order ``ic = nx*ny*k + nx*j + i``
and population order ``f[q*E + ic]``.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# src/input.hpp:221-256
CYCLIC, BOUNCEBACK, OUTLET, SYMMETRY, FIXEDVELOCITY, FIXEDDENSITY, WALLFUNCTION = 0, 1, 3, 4, 5, 6, 7
BC_NAMES = {"Cyclic": CYCLIC, "BounceBack": BOUNCEBACK, "Outlet": OUTLET, "Symmetry": SYMMETRY,
            "FixedVelocity": FIXEDVELOCITY, "FixedDensity": FIXEDDENSITY, "WallFunction": WALLFUNCTION}
FACES = ("nxMin", "nxMax", "nyMin", "nyMax", "nzMin", "nzMax")
SDF_NONE = np.float32(10000.0)  # ns.cpp:201


def lattice(q: int):
    """Velocity set and weights in the reference's population order.

    D3Q19: ``D3Q19_opencl/kernel.cl:3555-3560`` / ``D3Q19.hpp:9-27``.
    D3Q27: ``D3Q27_opencl/kernel.cl:2742-2747``.
    Returns (c[q,3] int, w[q] float32 rounded as the reference rounds them).
    """
    if q == 19:
        cx = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
        cy = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
        cz = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]
        w = [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12
    elif q == 27:
        cx = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, 1, -1]
        cy = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1, 1, -1]
        cz = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1, 1, -1, 1, -1, 1, -1, -1, 1]
        w = [8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8
    else:
        raise ValueError("q must be 19 or 27")
    c = np.stack([np.array(cx), np.array(cy), np.array(cz)], axis=1).astype(np.int64)
    return c, np.array(w, dtype=np.float32)


def opposite(q: int) -> np.ndarray:
    c, _ = lattice(q)
    out = np.empty(q, dtype=np.int64)
    for a in range(q):
        out[a] = int(np.nonzero((c == -c[a]).all(axis=1))[0][0])
    return out


@dataclass
class FaceBC:
    """Boundary settings of one domain face (``<face>Boundary1/2/3`` and ``<face>U0/V0/W0``)."""
    b1: int = CYCLIC
    b2: int = CYCLIC
    b3: int = CYCLIC
    u0: float = 0.0
    v0: float = 0.0
    w0: float = 0.0


@dataclass
class Case:
    """All per-cell inputs of one lattice case, in reference layout."""
    nx: int
    ny: int
    nz: int
    q: int = 19
    faces: dict = field(default_factory=dict)
    boundary: np.ndarray = None
    boundary1: np.ndarray = None
    boundary2: np.ndarray = None
    boundary3: np.ndarray = None
    u0: np.ndarray = None
    v0: np.ndarray = None
    w0: np.ndarray = None
    solid: np.ndarray = None
    nei_solid: np.ndarray = None
    sdf: np.ndarray = None
    omega: np.ndarray = None
    f: np.ndarray = None
    nu: float = 0.0

    @property
    def elements(self) -> int:
        return self.nx * self.ny * self.nz

    def arrays(self) -> dict:
        return {k: getattr(self, k) for k in ("boundary", "boundary1", "boundary2", "boundary3", "u0", "v0", "w0",
                                              "solid", "nei_solid", "sdf", "omega", "f")}


def omega_from_nu(nu: float) -> np.float32:
    """ns.cpp:127 ``omega0 = 1.0/(3.0*nu + 0.5)`` evaluated in double, stored as float."""
    return np.float32(1.0 / (3.0 * float(np.float32(nu)) + 0.5))


def face_arrays(nx, ny, nz, faces: dict):
    """boundary / boundary1-3 / u0-w0 exactly as setBoundaryConditions.hpp + ns.cpp:164-177."""
    E = nx * ny * nz
    fb = {name: faces.get(name, FaceBC()) for name in FACES}
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    b1 = np.zeros(E, np.int32)
    b2 = np.zeros(E, np.int32)
    b3 = np.zeros(E, np.int32)
    u0 = np.zeros(E, np.float32)
    v0 = np.zeros(E, np.float32)
    w0 = np.zeros(E, np.float32)

    def setv(mask, fc):
        u0[mask], v0[mask], w0[mask] = np.float32(fc.u0), np.float32(fc.v0), np.float32(fc.w0)

    xmin, xmax = (i == 0), (i == nx - 1) & (i != 0)
    ymin, ymax = (j == 0), (j == ny - 1) & (j != 0)
    zmin, zmax = (k == 0), (k == nz - 1) & (k != 0)
    b1[xmin] = fb["nxMin"].b1; setv(xmin, fb["nxMin"])
    b1[xmax] = fb["nxMax"].b1; setv(xmax, fb["nxMax"])
    b2[ymin] = fb["nyMin"].b2; setv(ymin, fb["nyMin"])
    b2[ymax] = fb["nyMax"].b2; setv(ymax, fb["nyMax"])
    b3[zmin] = fb["nzMin"].b3; setv(zmin, fb["nzMin"])
    b3[zmax] = fb["nzMax"].b3; setv(zmax, fb["nzMax"])

    f32 = np.float32
    nz1 = (nz - 1 != 0)

    def edge(mask, a, b, use_nz):
        for comp, arr in (("u0", u0), ("v0", v0), ("w0", w0)):
            va, vb = f32(getattr(a, comp)), f32(getattr(b, comp))
            zero = (f32(va * vb) == f32(0.0))
            if use_nz:
                zero = nz1 and zero
            arr[mask] = f32(0.0) if zero else va

    def corner(mask, a, b, c):
        for comp, arr in (("u0", u0), ("v0", v0), ("w0", w0)):
            va, vb, vc = f32(getattr(a, comp)), f32(getattr(b, comp)), f32(getattr(c, comp))
            zero = nz1 and (f32(f32(va * vb) * vc) == f32(0.0))
            arr[mask] = f32(0.0) if zero else va

    X0, X1, Y0, Y1, Z0, Z1 = (fb[n] for n in FACES)
    ie0, ie1 = (i == 0), (i == nx - 1)
    je0, je1 = (j == 0), (j == ny - 1)
    ke0, ke1 = (k == 0), (k == nz - 1)
    # setBoundaryConditions.hpp:56-78 (xy edges), 81-103 (xz), 106-128 (yz), 134-183 (corners); the later
    # rules overwrite the earlier ones cell by cell exactly as the sequential ifs do.
    edge(ie0 & je0, X0, Y0, False); edge(ie0 & je1, X0, Y1, False)
    edge(ie1 & je0, X1, Y0, False); edge(ie1 & je1, X1, Y1, False)
    edge(ie0 & ke0, X0, Z0, True); edge(ie0 & ke1, X0, Z1, True)
    edge(ie1 & ke0, X1, Z0, True); edge(ie1 & ke1, X1, Z1, True)
    edge(je0 & ke0, Y0, Z0, True); edge(je0 & ke1, Y0, Z1, True)
    edge(je1 & ke0, Y1, Z0, True); edge(je1 & ke1, Y1, Z1, True)
    corner(ie0 & je0 & ke0, X0, Y0, Z0); corner(ie1 & je0 & ke0, X1, Y0, Z0)
    corner(ie0 & je1 & ke0, X0, Y1, Z0); corner(ie0 & je0 & ke1, X0, Y0, Z1)
    corner(ie1 & je1 & ke0, X1, Y1, Z0); corner(ie0 & je1 & ke1, X0, Y1, Z1)
    corner(ie1 & je0 & ke1, X1, Y0, Z1); corner(ie1 & je1 & ke1, X1, Y1, Z1)

    face = (i == 0) | (i == nx - 1) | (j == 0) | (j == ny - 1)
    if nz - 1 != 0:
        face |= (k == 0) | (k == nz - 1)
    boundary = face.astype(np.int32)
    return boundary, b1, b2, b3, u0, v0, w0


def equilibrium(q, rho0, u, v, w, E):
    """initialization.hpp: f_q = (rho + 3 c.u + 4.5 (c.u)^2 - 1.5 u^2) w_q, in float."""
    c, wt = lattice(q)
    f32 = np.float32
    u, v, w = f32(u), f32(v), f32(w)
    out = np.empty((q, E), np.float32)
    usq = f32(f32(f32(u * u) + f32(v * v)) + f32(w * w))
    for a in range(q):
        udc = f32(f32(f32(u * f32(c[a, 0])) + f32(v * f32(c[a, 1]))) + f32(w * f32(c[a, 2])))
        val = f32(f32(f32(f32(rho0) + f32(f32(3.0) * udc)) + f32(f32(f32(4.5) * udc) * udc)) - f32(f32(1.5) * usq))
        out[a, :] = f32(val * wt[a])
    return out.ravel()


def nei_solid(solid: np.ndarray, nx, ny, nz, q) -> np.ndarray:
    """src/walls.hpp:187-216: fluid cells (not on a domain face unless that axis is 1 wide) with a solid
    upwind neighbour under periodic wrap (D3Q19.hpp ``upwindID``)."""
    c, _ = lattice(q)
    s = solid.reshape(nz, ny, nx).astype(bool)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    inner = ((nx == 1) & (j != 0) & (j != ny - 1) & (k != 0) & (k != nz - 1)) | \
            ((ny == 1) & (i != 0) & (i != nx - 1) & (k != 0) & (k != nz - 1)) | \
            ((nz == 1) & (i != 0) & (i != nx - 1) & (j != 0) & (j != ny - 1)) | \
            ((i != 0) & (i != nx - 1) & (j != 0) & (j != ny - 1) & (k != 0) & (k != nz - 1))
    hit = np.zeros_like(s)
    for a in range(q):
        up = np.roll(s, shift=(int(c[a, 2]), int(c[a, 1]), int(c[a, 0])), axis=(0, 1, 2))
        hit |= up
    out = inner & (~s) & hit
    return out.astype(np.uint8).ravel()


def make_case(nx, ny, nz, q=19, faces=None, nu=0.032, rho0=1.0, u_ini=(0.0, 0.0, 0.0), solid=None, sdf=None,
              omega=None) -> Case:
    """Assemble a case the way ns.cpp does, in lattice units (L = 1, c = 1)."""
    faces = faces or {}
    E = nx * ny * nz
    boundary, b1, b2, b3, u0, v0, w0 = face_arrays(nx, ny, nz, faces)
    if solid is None:
        solid = np.zeros(E, np.uint8)
    solid = np.ascontiguousarray(solid, dtype=np.uint8)
    ns = nei_solid(solid, nx, ny, nz, q)
    if sdf is None:
        sdf = np.full(E, SDF_NONE, np.float32)
    if omega is None:
        omega = np.full(E, omega_from_nu(nu), np.float32)
    f = equilibrium(q, rho0, *u_ini, E)
    return Case(nx, ny, nz, q, dict(faces), boundary, b1, b2, b3, u0, v0, w0, solid, ns,
                np.ascontiguousarray(sdf, dtype=np.float32), np.ascontiguousarray(omega, dtype=np.float32), f, nu)


def cavity_faces(u_lid=0.05):
    """Lid-driven cavity: five BounceBack faces and a FixedVelocity lid at nyMax (testCases/cavityFlow)."""
    return {"nxMin": FaceBC(BOUNCEBACK, CYCLIC, CYCLIC), "nxMax": FaceBC(BOUNCEBACK, CYCLIC, CYCLIC),
            "nyMin": FaceBC(CYCLIC, BOUNCEBACK, CYCLIC), "nyMax": FaceBC(CYCLIC, FIXEDVELOCITY, CYCLIC, u_lid, 0, 0),
            "nzMin": FaceBC(CYCLIC, CYCLIC, BOUNCEBACK), "nzMax": FaceBC(CYCLIC, CYCLIC, BOUNCEBACK)}


def channel_faces(u_in=0.05, top_bottom=SYMMETRY, z_periodic=True):
    """Channel: FixedVelocity inlet at nxMin, Geier Outlet at nxMax, y faces Symmetry (or walls), z Cyclic."""
    z = CYCLIC if z_periodic else BOUNCEBACK
    return {"nxMin": FaceBC(FIXEDVELOCITY, CYCLIC, CYCLIC, u_in, 0, 0), "nxMax": FaceBC(OUTLET, CYCLIC, CYCLIC),
            "nyMin": FaceBC(CYCLIC, top_bottom, CYCLIC), "nyMax": FaceBC(CYCLIC, top_bottom, CYCLIC),
            "nzMin": FaceBC(CYCLIC, CYCLIC, z), "nzMax": FaceBC(CYCLIC, CYCLIC, z)}
