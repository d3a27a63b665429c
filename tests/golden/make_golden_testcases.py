"""Extract the physics fixtures of the reference's own test cases into tests/golden/testcases.npz.

The reference ships results of three of its test cases as plain data next to their inputs
(testCases/<case>/input.txt, boundaryConditions.txt):

* cavityFlow/u_x05.csv          u along the vertical centre line x = 0.5 of the 100x100x1 lid-driven
                                cavity at Re 100 (its endTimeStep), as exported from its VTK output;
* poiseuilleFlow/u.csv          u across the 100x20x1 pressure-gradient-driven channel;
* flowAroundCylinder/t_Cx.dat,  drag and lift coefficients of the 1200x400x1 channel with a cylinder
  t_Cy.dat                      (D = 0.1, Re 100), one sample per output interval (t in seconds).

This script keeps the columns the regression tests compare (sorted by position or time), the
input.txt parameters of each case, and the cylinder's centre and radius measured from the case's
cylinder.stl (its vertices' bounding box and radial extent), so the tests need nothing from the
reference checkout at run time.  Third-party comparison data shipped beside them (Ghia.dat) is not
read.

usage: python tests/golden/make_golden_testcases.py --lbffs <reference checkout>
       (or set LBFFS_REFERENCE)
"""
import argparse
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_input(path):
    """key -> value of an input.txt (src/input.hpp reads the same 'key value' lines; a trailing 'f' on a
    number is ignored as the reference's stof ignores it)."""
    out = {}
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2:
            try:
                out[parts[0]] = float(parts[1].rstrip("f"))
            except ValueError:
                out[parts[0]] = parts[1]
    return out


def read_csv(path, cols):
    d = np.genfromtxt(path, delimiter=",", names=True)
    return {c: np.asarray(d[c.replace(":", "")], dtype=np.float64) for c in cols}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--lbffs", default=os.environ.get("LBFFS_REFERENCE"),
                    help="the reference checkout (its testCases directory is read)")
    args = ap.parse_args()
    if not args.lbffs:
        ap.error("give the reference checkout with --lbffs or LBFFS_REFERENCE")
    tc = os.path.join(args.lbffs, "testCases")
    out = {}
    keys = ("nx", "ny", "nz", "Lx", "uMax", "U0", "nu", "dpdx", "endTimeStep", "outInterval")

    p = read_input(os.path.join(tc, "cavityFlow", "input.txt"))
    d = read_csv(os.path.join(tc, "cavityFlow", "u_x05.csv"), ["u", "Points:0", "Points:1"])
    o = np.argsort(d["Points:1"])
    out["cavity_y"], out["cavity_u"], out["cavity_x"] = d["Points:1"][o], d["u"][o], d["Points:0"][o]
    out["cavity_params"] = np.array([p[k] for k in keys])

    p = read_input(os.path.join(tc, "poiseuilleFlow", "input.txt"))
    d = read_csv(os.path.join(tc, "poiseuilleFlow", "u.csv"), ["u", "Points:0", "Points:1"])
    o = np.argsort(d["Points:1"])
    out["pois_y"], out["pois_u"], out["pois_x"] = d["Points:1"][o], d["u"][o], d["Points:0"][o]
    out["pois_params"] = np.array([p[k] for k in keys])

    p = read_input(os.path.join(tc, "flowAroundCylinder", "input.txt"))
    cx = np.loadtxt(os.path.join(tc, "flowAroundCylinder", "t_Cx.dat"))
    cy = np.loadtxt(os.path.join(tc, "flowAroundCylinder", "t_Cy.dat"))
    out["cyl_t"], out["cyl_cx"], out["cyl_cy"] = cx[:, 0], cx[:, 1], cy[:, 1]
    out["cyl_params"] = np.array([p[k] for k in keys] + [p["Dref"]])
    txt = open(os.path.join(tc, "flowAroundCylinder", "cylinder.stl")).read()
    v = np.array(re.findall(r"vertex\s+(\S+)\s+(\S+)\s+(\S+)", txt), dtype=np.float64)
    centre = 0.5 * (v.min(0) + v.max(0))
    out["cyl_stl_centre_radius"] = np.array([centre[0], centre[1], np.hypot(v[:, 0] - centre[0],
                                                                           v[:, 1] - centre[1]).max()])
    out["param_keys"] = np.array(keys)
    np.savez_compressed(os.path.join(HERE, "testcases.npz"), **out)
    print("wrote", os.path.join(HERE, "testcases.npz"))


if __name__ == "__main__":
    main()
