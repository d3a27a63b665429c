"""Procedural geometry for the synthetic workloads.

The reference voxelises ASCII STL files on the host (``src/walls.hpp``,
``src/stl.hpp``).  The benchmark and test workloads here are seeded synthetic
shapes: analytic solid masks with analytic signed distances (positive in the
fluid, lattice units, ``10000`` = not set as in ``ns.cpp:201``), and an ASCII
STL writer for a seeded closed triangle mesh (used to pin the reference's own
voxeliser output).
"""
from __future__ import annotations

import re
from fractions import Fraction

import numpy as np

SDF_NONE = np.float32(10000.0)


def _grid(nx, ny, nz):
    k, j, i = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    return i, j, k


def cylinder_z(nx, ny, nz, cx, cy, radius, sdf_band=10.0):
    """Cylinder along z centred at (cx, cy): solid mask and signed distance (fluid > 0) within sdf_band."""
    i, j, _ = _grid(nx, ny, nz)
    d = np.sqrt((i - cx) ** 2 + (j - cy) ** 2) - radius
    solid = (d < 0).astype(np.uint8).ravel()
    sdf = d.astype(np.float32).ravel()
    sdf[np.abs(sdf) > sdf_band] = SDF_NONE
    return solid, sdf


def ellipsoid(nx, ny, nz, center, radii, sdf_band=10.0):
    """Ellipsoid body: solid mask and an approximate signed distance (fluid > 0) within sdf_band,
    (|x / r| - 1) scaled by the smallest radius (exact on the sphere, first order elsewhere)."""
    i, j, k = _grid(nx, ny, nz)
    rr = np.sqrt(((i - center[0]) / radii[0]) ** 2 + ((j - center[1]) / radii[1]) ** 2 +
                 ((k - center[2]) / radii[2]) ** 2)
    d = (rr - 1.0) * min(radii)
    solid = (d < 0).astype(np.uint8).ravel()
    sdf = d.astype(np.float32).ravel()
    sdf[np.abs(sdf) > sdf_band] = SDF_NONE
    return solid, sdf


def backward_step(nx, ny, nz, x_end, height, sdf_band=3.0):
    """Solid block j < height for i < x_end (backward-facing step); distance to the block's faces."""
    i, j, _ = _grid(nx, ny, nz)
    solid = ((i < x_end) & (j < height)).astype(np.uint8).ravel()
    dx = i - (x_end - 0.5)
    dy = j - (height - 0.5)
    outside = np.where(i < x_end, dy, np.where(j < height, dx, np.sqrt(np.maximum(dx, 0) ** 2 + np.maximum(dy, 0) ** 2)))
    inside = -np.minimum(-dx, -dy)
    d = np.where(solid.reshape(i.shape) == 1, inside, outside)
    sdf = d.astype(np.float32).ravel()
    sdf[np.abs(sdf) > sdf_band] = SDF_NONE
    return solid, sdf


def ellipsoid_mesh(seed, n_theta, n_phi, center, radii, noise=0.05):
    """Closed triangle mesh of a noisy ellipsoid (2*n_phi*(n_theta-1) triangles), seeded radial noise."""
    rng = np.random.default_rng(seed)
    th = np.linspace(0.0, np.pi, n_theta + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, n_phi, endpoint=False)
    scale = 1.0 + noise * (2.0 * rng.random((n_theta + 1, n_phi)) - 1.0)
    scale[0, :] = scale[0, 0]
    scale[-1, :] = scale[-1, 0]
    T, P = np.meshgrid(th, ph, indexing="ij")
    pts = np.stack([np.sin(T) * np.cos(P) * radii[0], np.sin(T) * np.sin(P) * radii[1], np.cos(T) * radii[2]], -1)
    pts = pts * scale[..., None] + np.asarray(center, dtype=np.float64)
    tris = []
    for a in range(n_theta):
        for b in range(n_phi):
            b1 = (b + 1) % n_phi
            p00, p01, p10, p11 = pts[a, b], pts[a, b1], pts[a + 1, b], pts[a + 1, b1]
            if a > 0:
                tris.append((p00, p10, p01))
            if a < n_theta - 1:
                tris.append((p01, p10, p11))
    return np.array(tris)


def facet_normals(tris):
    """Unit normals (v1 - v0) x (v2 - v0) of (ntri, 3, 3) triangles, in float64 (zero for a
    degenerate triangle)."""
    t = np.asarray(tris, dtype=np.float64)
    n = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(ln > 0, n / np.where(ln > 0, ln, 1.0), n)


def write_ascii_stl(path, tris, name="walls"):
    """ASCII STL in the layout src/stl.hpp:18-83 parses (one leading blank on vertex lines).
    ``tris`` is one (ntri, 3, 3) array, or a list of (name, tris) pairs written as patches."""
    patches = tris if isinstance(tris, list) else [(name, tris)]
    with open(path, "w") as fh:
        for pname, ptris in patches:
            fh.write(f"solid {pname}\n")
            for t, n in zip(ptris, facet_normals(ptris)):
                fh.write(f"  facet normal {n[0]:.6e} {n[1]:.6e} {n[2]:.6e}\n    outer loop\n")
                for v in t:
                    fh.write(f"      vertex {v[0]:.6e} {v[1]:.6e} {v[2]:.6e}\n")
                fh.write("    endloop\n  endfacet\n")
            fh.write(f"endsolid {pname}\n")


def _stof(tok):
    """The float32 nearest to the decimal text (ties to even), as std::stof rounds it."""
    x = Fraction(tok)
    f = np.float32(float(x))
    cands = (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf)))
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - x), int(np.float32(c).view(np.uint32)) & 1))


def read_ascii_stl(path, L=1.0):
    """Triangles of an ASCII STL as src/stl.hpp:455-523 reads them: the tokens of readToLines
    (src/input.hpp:90-110, each line split at runs of blanks, so an indented line starts with an
    empty token), the facets assigned to patches as stl.hpp assigns them, std::stof of each number, vertices divided by L (normalizeSTLv).  Returns (vertices
    (ntri, 3, 3) float32, normals (ntri, 3) float32, triangles per patch)."""
    with open(path, newline="\n") as fh:
        lines = fh.read().split("\n")
    if lines and lines[-1] == "":  # std::getline yields no line after the final newline
        lines.pop()
    toks = [t for line in lines for t in re.split(r"\s+", line)]
    # one patch per "solid" token (stl.hpp:477-483); facets go to the current patch, which advances
    # at a "solid" token naming another patch (stl.hpp:486-495)
    names = [toks[i + 1] if i + 1 < len(toks) else "" for i, t in enumerate(toks) if t == "solid"]
    counts, verts, norms = [0] * len(names), [], []
    cur = 0
    i = 0
    while i < len(toks):
        t = toks[i]
        if t == "solid":
            if toks[i + 1] != names[cur]:
                cur += 1
                i += 1
        elif t == "facet":
            norms.append([_stof(toks[i + 2]), _stof(toks[i + 3]), _stof(toks[i + 4])])
            i += 4
        elif t == "vertex":
            tri = []
            for _ in range(3):
                tri.append([_stof(toks[i + 1]), _stof(toks[i + 2]), _stof(toks[i + 3])])
                i += 5
            i -= 2
            verts.append(tri)
            counts[cur] += 1
        i += 1
    v = np.array(verts, dtype=np.float32).reshape(-1, 3, 3) / np.float32(L)
    n = np.array(norms, dtype=np.float32).reshape(-1, 3)
    return v.astype(np.float32), n, counts


def cylinder_markers(n, cx, cy, cz, radius):
    """IBM markers on a circle of the given radius (a cylinder cross-section) at height cz."""
    t = 2.0 * np.pi * np.arange(n) / n
    return np.stack([cx + radius * np.cos(t), cy + radius * np.sin(t), np.full(n, cz)], 1).astype(np.float32)
