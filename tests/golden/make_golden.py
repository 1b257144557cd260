"""Generate the golden fixtures from the reference solver itself.

Runs every case in ``cases.py`` through ``oracle/_ref/libref.so`` -- the
lbm-2d reference headers compiled unmodified by ``oracle/Makefile`` (target
``ref``) -- and writes ``tests/golden/<case>.npz`` with the solid mask, the
final populations (f, and g for thermal cases), the per-node momentum-exchange
force fields, the per-step driver force sums and, for LES cases, the wall
distance.  ``kat.npz`` holds known-answer vectors for the geometry helpers.

Usage (in a container that has the reference sources):
    make -C oracle ref REF_SRC=<lbm-2d>/src
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import cases as CS  # noqa: E402


def run_case(kind: str, spec: dict) -> dict:
    s = O.Solver(spec["nx"], spec["ny"], kind)
    CS.apply_setup(s, spec,
                   naca_fn=lambda ser, n: O.naca_coords(ser, n, kind),
                   transform_fn=lambda p, *a: O.transform_points(p, *a, kind=kind))
    out = {"mask": s.obstacle.copy()}
    th = spec.get("thermal")
    hook = th.get("hook") if th else None
    sums = []
    for _ in range(spec["steps"]):
        s.step(spec["tau"], spec["u"])
        if hook:
            s.thermal_hook(*hook)
        sums.append(s.force_sums())
    out["f"] = s.f.copy()
    if th:
        out["g"] = s.g.copy()
    out["fx"] = s.fx.copy()
    out["fy"] = s.fy.copy()
    out["sums"] = np.array(sums, np.float64)
    if spec.get("les"):
        out["wall_dist"] = s.wall_dist.copy()
    s.close()
    return out


def kat(kind: str) -> dict:
    out = {}
    for series, n in ((12, 50), (2412, 60), (4415, 33)):
        out[f"naca_{series}_{n}"] = O.naca_coords(series, n, kind)
    p = O.naca_coords(2412, 40, kind)
    out["transform_2412"] = O.transform_points(p, 30.0, 20.0, 36.0, 8.0, kind)
    poly = out["transform_2412"]
    pts = [(x + 0.25, y + 0.5) for x in range(24, 70, 3) for y in range(10, 32, 2)]
    out["pip"] = np.array([O.point_in_polygon(x, y, poly, kind) for x, y in pts], np.uint8)
    out["pip_pts"] = np.array(pts, np.float64)
    eq = []
    for rho, u, v in ((1.0, 0.0, 0.0), (1.2, 0.1, 0.05), (1.5, 0.12, -0.08), (0.9, -0.07, 0.11)):
        eq.append([O.equilibrium(i, rho, u, v, kind) for i in range(9)])
    out["equilibrium"] = np.array(eq)
    # interpolated bounce-back distances for a circle and a polygon
    s = O.Solver(48, 40, kind)
    s.place_cylinder(20, 21, 7)
    qs = [s.compute_q(x, y, i) for x in range(10, 31) for y in range(11, 32) for i in range(9)]
    out["q_cylinder"] = np.array(qs)
    s.close()
    s = O.Solver(96, 40, kind)
    s.place_polygon(poly)
    qs = [s.compute_q(x, y, i) for x in range(26, 70, 2) for y in range(14, 28) for i in range(9)]
    out["q_polygon"] = np.array(qs)
    s.close()
    return out


def run_ibm_case(kind: str, spec: dict) -> dict:
    """The airfoil immersed-boundary driver loop (src/airfoil_ibm.cpp:121-176)
    on the reference's ImmersedBoundary (kind "ref") or the restatement."""
    s = O.Solver(spec["nx"], spec["ny"], kind)
    poly = CS.ibm_setup(s, spec,
                        naca_fn=lambda ser, n: O.naca_coords(ser, n, kind),
                        transform_fn=lambda p, *a: O.transform_points(p, *a, kind=kind),
                        pip_fn=lambda x, y, p: O.point_in_polygon(x, y, p, kind),
                        eq_fn=lambda i, r, u, v: O.equilibrium(i, r, u, v, kind))
    out = {"mask": s.obstacle.copy(), "f0": s.f.copy(), "poly": poly}
    out["points"] = s.ibm_from_polygon(poly, spec["spacing"])
    tau = CS.ibm_tau(spec)
    sums = []
    for _ in range(spec["steps"]):
        s.ibm_step(tau, spec["u"])
        sums.append(s.force_sums())
    out["f"] = s.f.copy()
    out["U"], out["V"], out["FX"], out["FY"] = s.ibm_lagrangian()
    out["sums"] = np.array(sums, np.float64)
    s.close()
    return out


def main():
    if not os.path.exists(O.LIB_REF):
        sys.exit("oracle/_ref/libref.so missing: build it with `make -C oracle ref`")
    for name, spec in CS.CASES.items():
        res = run_case("ref", spec)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
        print(f"{name}: steps={spec['steps']} sums[-1]={res['sums'][-1]}")
    for name, spec in CS.IBM_CASES.items():
        res = run_ibm_case("ref", spec)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **res)
        print(f"{name}: points={len(res['points'])} steps={spec['steps']}")
    np.savez_compressed(os.path.join(HERE, "kat.npz"), **kat("ref"))
    print("kat written")


if __name__ == "__main__":
    main()
