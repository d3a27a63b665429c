"""CPU restatement of the LES wall-distance set-up (numpy).

Test infrastructure only: the check for ``lbffs_build_sdf``.  Follows
``src/walls.hpp:218-268`` (setSDF: near box around neiSolid cells, inverse-distance-weighted
signed distance over the triangles closer than dr, in triangle order) and
``src/walls.hpp:372-467`` (setSDFnearBwalls), called as ``D3Q19_opencl/ns.cpp:200-225`` calls
them (setSDF once per patch, then the face pass).

The expression types are those the reference's host compiler gives them: ``pow`` and ``sqrt``
there are the C library's double functions, so the squared offsets, their sum and the square root
are double (r is then stored as float), the weight r^-p and the products sd * r^-p are double, and
each ``+=`` adds in double before storing float.  The offsets and sd are float arithmetic.
"""
from __future__ import annotations

import numpy as np


def near_cells(nei, nx, ny, nz, dr):
    """Cells within a Chebyshev box of half-width int(dr) around a neiSolid cell (walls.hpp:223-257)."""
    r = int(dr)
    m = nei.reshape(nz, ny, nx) == 1
    for ax in (2, 1, 0):
        out = np.zeros_like(m)
        n = m.shape[ax]
        for d in range(-r, r + 1):
            lo, hi = max(0, -d), min(n, n - d)  # out[x] |= m[x + d] for 0 <= x + d < n
            if lo >= hi:
                continue
            src = [slice(None)] * 3
            dst = [slice(None)] * 3
            src[ax] = slice(lo + d, hi + d)
            dst[ax] = slice(lo, hi)
            out[tuple(dst)] |= m[tuple(src)]
        m = out
    return np.flatnonzero(m.reshape(-1))


def centroids(vertices):
    """((v0 + v1) + v2) / 3 in float32 (stl.hpp:177-186)."""
    v = vertices.astype(np.float32)
    return ((v[:, 0] + v[:, 1]) + v[:, 2]) / np.float32(3.0)


def set_sdf(sdf, sdf_ini, dr, p, cen, nrm, nx, ny, nz, nei, cells=None):
    """setSDF of one patch (walls.hpp:218-268), in place; ``cells`` restricts the near cells
    evaluated (a subset of a large case)."""
    near = near_cells(nei, nx, ny, nz, dr)
    if cells is not None:
        near = np.intersect1d(near, cells)
    drf = np.float32(dr)
    mp = -float(np.float32(p))
    for ic in near:
        i, j, k = ic % nx, (ic // nx) % ny, ic // (nx * ny)
        dx = np.float32(i) - cen[:, 0]
        dy = np.float32(j) - cen[:, 1]
        dz = np.float32(k) - cen[:, 2]
        ddx, ddy, ddz = dx.astype(np.float64), dy.astype(np.float64), dz.astype(np.float64)
        r = np.sqrt((ddx * ddx + ddy * ddy) + ddz * ddz).astype(np.float32)
        sel = np.flatnonzero(r < drf)
        s = np.float32(0.0)
        a = np.float32(0.0)
        if sel.size:
            sd = (dx[sel] * nrm[sel, 0] + dy[sel] * nrm[sel, 1]) + dz[sel] * nrm[sel, 2]
            w = np.power(r[sel].astype(np.float64), mp)
            sdw = sd.astype(np.float64) * w
            for t in range(sel.size):
                s = np.float32(np.float64(s) + w[t])
                a = np.float32(np.float64(a) + sdw[t])
        sdf[ic] = a / s if s != 0 else np.float32(sdf_ini)


def set_sdf_near_bwalls(sdf, dr, b1, b2, b3, nx, ny, nz):
    """setSDFnearBwalls (walls.hpp:372-467), the loops in the reference's order."""
    s = sdf.reshape(nz, ny, nx)
    B1, B2, B3 = (b.reshape(nz, ny, nx) for b in (b1, b2, b3))
    n = int(dr) + 1
    half = np.float32(0.5)
    for k in range(nz):
        for j in range(ny):
            if B1[k, j, 0] == 1:
                for i in range(n):
                    if i < nx - 1:
                        s[k, j, i] = half + np.float32(i)
            if B1[k, j, nx - 1] == 1:
                for i in range(n):
                    if nx - 1 - i > 0:
                        s[k, j, nx - 1 - i] = half + np.float32(i)
    for k in range(nz):
        for i in range(nx):
            if B2[k, 0, i] == 1:
                for j in range(n):
                    if j < ny - 1:
                        s[k, j, i] = half + np.float32(j)
            if B2[k, ny - 1, i] == 1:
                for j in range(n):
                    if ny - 1 - j > 0:
                        s[k, ny - 1 - j, i] = half + np.float32(j)
    for j in range(ny):
        for i in range(nx):
            if B3[0, j, i] == 1:
                for k in range(n):
                    if k < nz - 1:
                        s[k, j, i] = half + np.float32(k)
            if B3[nz - 1, j, i] == 1:
                for k in range(n):
                    if nz - 1 - k > 0:
                        s[nz - 1 - k, j, i] = half + np.float32(k)


def les_sdf(vertices, normals, patch_ntri, nei, b1, b2, b3, nx, ny, nz, dr=10.0, p=7.0, sdf_ini=10000.0,
            dr_walls=3.0, cells=None):
    """The sequence of ns.cpp:200-225: sdf = sdfIni, setSDF per patch, setSDFnearBwalls."""
    sdf = np.full(nx * ny * nz, np.float32(sdf_ini), dtype=np.float32)
    cen = centroids(vertices)
    nrm = normals.astype(np.float32)
    t0 = 0
    for cnt in patch_ntri:
        set_sdf(sdf, sdf_ini, dr, p, cen[t0:t0 + cnt], nrm[t0:t0 + cnt], nx, ny, nz, nei, cells)
        t0 += cnt
    if dr_walls is not None and int(dr_walls) >= 0:
        set_sdf_near_bwalls(sdf, dr_walls, b1, b2, b3, nx, ny, nz)
    return sdf
