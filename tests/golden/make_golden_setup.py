"""Record golden vectors of the reference's host setup (run here, on the CPU).

* face boundary arrays from src/setBoundaryConditions.hpp (+ the face flag of
  ns.cpp:164-177) via oracle/_ref/case_ref, for several face settings;
* voxelised solid / neiSolid / sdf from src/walls.hpp + src/stl.hpp via
  oracle/_ref/voxel_ref19 / voxel_ref27 for seeded synthetic STL meshes.

usage: python tests/golden/make_golden_setup.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.path.join(ROOT, "oracle", "_ref")

from lbffs_gb300 import geometry as G  # noqa: E402

FACE_SETS = {
    "cavity": [(1, 0, 0, 0, 0, 0), (1, 0, 0, 0, 0, 0), (0, 1, 0, 0, 0, 0), (0, 5, 0, 0.05, 0, 0), (0, 0, 1, 0, 0, 0),
               (0, 0, 1, 0, 0, 0)],
    "channel": [(5, 0, 0, 0.05, 0, 0), (3, 0, 0, 0, 0, 0), (0, 4, 0, 0, 0, 0), (0, 4, 0, 0, 0, 0), (0, 0, 0, 0, 0, 0),
                (0, 0, 0, 0, 0, 0)],
    "moving_edges": [(5, 0, 0, 0.04, 0.01, -0.02), (6, 0, 0, 0, 0, 0), (0, 5, 0, 0.03, 0.02, 0.0),
                     (0, 5, 0, 0.05, -0.01, 0.01), (0, 0, 5, 0.02, 0.03, 0.04), (0, 0, 1, 0, 0, 0)],
}
FACE_GRIDS = [(9, 7, 6), (10, 8, 1)]


def faces():
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, fs in FACE_SETS.items():
            for (nx, ny, nz) in FACE_GRIDS:
                args = [os.path.join(REF, "case_ref"), str(nx), str(ny), str(nz)]
                for f in fs:
                    args += [str(v) for v in f]
                pre = os.path.join(td, "o_")
                subprocess.run(args + [pre], check=True)
                key = f"{name}_{nx}x{ny}x{nz}"
                for fld, dt in (("boundary", np.int32), ("boundary1", np.int32), ("boundary2", np.int32),
                                ("boundary3", np.int32), ("u0", np.float32), ("v0", np.float32), ("w0", np.float32)):
                    ext = "i32" if dt == np.int32 else "f32"
                    out[f"{key}__{fld}"] = np.fromfile(pre + f"{fld}.{ext}", dtype=dt)
    np.savez_compressed(os.path.join(HERE, "setup_faces.npz"), **out)


VOXEL_CASES = {
    # name: (q, nx, ny, nz, mesh builder[, invertFluidSolid])
    "ellipsoid_q19": (19, 40, 32, 30, lambda: G.ellipsoid_mesh(7, 18, 36, (19.3, 15.6, 14.8), (11.0, 8.0, 7.5))),
    "ellipsoid_q27": (27, 40, 32, 30, lambda: G.ellipsoid_mesh(11, 18, 36, (20.1, 16.2, 15.1), (12.0, 9.0, 8.0))),
    "ellipsoid_big_q19": (19, 96, 80, 72,
                          lambda: G.ellipsoid_mesh(23, 40, 80, (47.7, 39.2, 35.6), (30.0, 22.0, 20.5), noise=0.05)),
    "ellipsoid_inv_q19": (19, 40, 32, 30, lambda: G.ellipsoid_mesh(31, 18, 36, (19.1, 15.9, 14.6), (13.0, 10.0, 9.0)),
                          1),
    # two STL patches (setSDF runs once per patch) and bounce-back codes on other faces
    "two_patch_q19": (19, 36, 28, 26, lambda: [("front", G.ellipsoid_mesh(41, 12, 24, (11.2, 13.7, 12.9), (6.0, 5.0, 5.5))),
                                               ("back", G.ellipsoid_mesh(43, 12, 24, (24.6, 14.1, 13.3), (5.5, 6.5, 5.0)))],
                      0, (0, 1, 1, 0, 1, 1)),
}

# face BC codes (x min, x max, y min, y max, z min, z max) of the voxel cases unless given
VOXEL_BC = (1, 1, 1, 1, 0, 0)


def voxels():
    out = {}
    with tempfile.TemporaryDirectory() as td:
        for name, spec in VOXEL_CASES.items():
            q, nx, ny, nz, mesh = spec[:5]
            invert = spec[5] if len(spec) > 5 else 0
            bc = spec[6] if len(spec) > 6 else VOXEL_BC
            stl = os.path.join(td, "walls.stl")
            G.write_ascii_stl(stl, mesh())
            pre = os.path.join(td, "v_")
            # face codes as setSDFnearBwalls sees them (1 = BounceBack); withSDF on
            subprocess.run([os.path.join(REF, f"voxel_ref{q}"), stl, str(nx), str(ny), str(nz), "1.0", str(invert),
                            "1"] + [str(b) for b in bc] + [pre], check=True, stdout=subprocess.DEVNULL)
            out[f"{name}__solid"] = np.fromfile(pre + "solid.u8", dtype=np.uint8)
            out[f"{name}__nei_solid"] = np.fromfile(pre + "neiSolid.u8", dtype=np.uint8)
            out[f"{name}__sdf"] = np.fromfile(pre + "sdf.f32", dtype=np.float32)
            out[f"{name}__shape"] = np.array([q, nx, ny, nz])
            out[f"{name}__invert"] = np.array([invert])
            out[f"{name}__bc"] = np.array(bc)
            print(name, int(out[f"{name}__solid"].sum()), "solid cells,", int(out[f"{name}__nei_solid"].sum()),
                  "neiSolid cells")
    np.savez_compressed(os.path.join(HERE, "setup_voxels.npz"), **out)


if __name__ == "__main__":
    faces()
    voxels()
