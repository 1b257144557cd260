"""Configure a product Solver exactly like a golden case.

The oracle runs the case's set-up (driver geometry, seeded initial state,
one-off thermal passes); the product solver then receives the same mask, the
same bounce-back geometry parameters and the same initial populations through
its public API.  Test infrastructure only."""
import numpy as np

import cases as CS


def oracle_setup(O, spec):
    s = O.Solver(spec["nx"], spec["ny"], "oracle")
    CS.apply_setup(s, spec, naca_fn=O.naca_coords, transform_fn=O.transform_points)
    return s


def gpu_solver(lbm2d, O, spec, storage="fp32"):
    s = oracle_setup(O, spec)
    mask, f0 = s.obstacle.copy(), s.f.copy()
    th = spec.get("thermal")
    g0 = s.g.copy() if th else None
    s.close()
    g = lbm2d.Solver(spec["nx"], spec["ny"], spec["case"], spec.get("collision", 0), spec.get("les", False),
                     spec.get("cs", 0.12), storage)
    g.set_mask(mask)
    for op in spec["geometry"]:  # bb_geom keeps the last circle / polygon
        if op[0] == "cylinder":
            g.set_bb_cylinder(*op[1:])
        elif op[0] in ("polygon", "naca"):
            g.set_bb_polygon(CS.polygon_of(op, O.naca_coords, O.transform_points))
    if "moving_wall" in spec:
        g.set_moving_wall(True, *spec["moving_wall"])
    if not spec.get("mei", True):
        g.set_mei(False)
    if spec.get("body_force"):
        g.set_body_force(spec["body_force"])
    if th:
        g.set_thermal(True, th["T_ref"], th["alpha"], th["omega_k"], th["beta"], th["g_buoyancy"])
        if th.get("hook"):
            g.set_thermal_hook(*th["hook"])
        g.upload_g(g0)
    g.upload_f(f0)
    return g


def rel_l2(a, b, mask=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def fluid_pop_mask(mask):
    return np.repeat(mask == 0, 9)


def velocity(f):
    f = f.reshape(-1, 9)
    cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], np.float64)
    cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], np.float64)
    rho = f.sum(1)
    with np.errstate(invalid="ignore", divide="ignore"):
        return (f @ cx) / rho, (f @ cy) / rho
