"""Case specifications shared by the fixture generator and the parity tests.

A case is a plain dict: grid, reference case type, collision, LES, geometry
operations (applied in order, as the reference drivers do), the initial
state, optional thermal setup with the drivers' post-step thermal pass,
and the (tau, u) pair passed to every step.

``apply_setup(target, spec)`` drives anything with the oracle's Solver
surface (place_walls, place_cylinder, obstacle view, init_* ...).  The GPU
tests use the same specs through the product's own API.
"""
from __future__ import annotations

import math

import numpy as np

CYLINDER, CAVITY, STEP, RIBS, URBAN_CANYON, DOWNWASH, SQUARE_CYLINDER, FLAT_PLATE, \
    SPORTS_BALL, PERIODIC_HILLS, CYLINDER_NEAR_WALL, SIDE_BY_SIDE, ROTATING_CYLINDER, \
    ORIFICE_PLATE = range(14)
MRT, BGK = 0, 1


def step_mask(nx, ny):
    """Backward-facing step geometry of src/step.cpp:89-104 (h = NY/3)."""
    m = np.zeros((ny, nx), np.uint8)
    m[0, :] = 1
    m[ny - 1, :] = 1
    m[: ny // 3, : nx // 4] = 1
    return m.reshape(-1)


def hills_mask(nx, ny, hmax_frac=1.0 / 6.0):
    """Periodic-hills geometry of src/periodic_hills.cpp:95-113 (3 cycles, L = NX)."""
    H = ny * 2 // 3
    h_max = max(1, int(H * hmax_frac))
    m = np.zeros((ny, nx), np.uint8)
    for x in range(nx):
        xr = x / nx * 3
        hy = H - h_max * 0.5 * (1.0 - math.cos(2.0 * math.pi * xr)) * (1.0 - math.cos(2.0 * math.pi * xr))
        iy = int(math.ceil(hy))
        m[ny - 1, x] = 1
        m[:max(0, min(iy, ny)), x] = 1
    return m.reshape(-1)


def channel_circles_mask(nx, ny, n_circles, rmin, rmax, seed):
    """Periodic-x channel with solid rows y=0, y=NY-1 and seeded non-overlapping
    circles (the large-domain workload).  Circles use the reference's
    place_cylinder rule sqrt(dx^2+dy^2) < r on integer centres."""
    rng = np.random.default_rng(seed)
    m = np.zeros((ny, nx), np.uint8)
    m[0, :] = 1
    m[ny - 1, :] = 1
    circles = []
    tries = 0
    while len(circles) < n_circles and tries < 100000:
        tries += 1
        r = int(rng.integers(rmin, rmax + 1))
        cx = int(rng.integers(r + 2, nx - r - 2))
        cy = int(rng.integers(r + 3, ny - r - 3))
        if all((cx - a) ** 2 + (cy - b) ** 2 > (r + c + 3) ** 2 for a, b, c in circles):
            circles.append((cx, cy, r))
    for cx, cy, r in circles:
        # only the circle's bounding box can hold nodes with d < r
        y0, y1, x0, x1 = max(cy - r, 0), min(cy + r + 1, ny), max(cx - r, 0), min(cx + r + 1, nx)
        yy, xx = np.mgrid[y0:y1, x0:x1]
        d = np.sqrt(((xx - cx).astype(np.float64)) ** 2 + ((yy - cy).astype(np.float64)) ** 2)
        m[y0:y1, x0:x1][d < r] = 1
    return m.reshape(-1), circles


def square_poly(cx, cy, half):
    return np.array([[cx - half, cy - half], [cx + half, cy - half],
                     [cx + half, cy + half], [cx - half, cy + half]], np.float64)


# --------------------------------------------------------------------------- cases

CASES = {
    "cavity_mrt": dict(nx=40, ny=32, case=CAVITY, collision=MRT, tau=0.68, u=0.1, steps=60,
                       geometry=[("walls",)], init=("uniform", 1.0, 0.0, 0.0)),
    "cavity_bgk": dict(nx=36, ny=28, case=CAVITY, collision=BGK, tau=0.62, u=0.1, steps=50,
                       geometry=[("walls",)], init=("uniform", 1.0, 0.0, 0.0)),
    "cavity_les": dict(nx=32, ny=32, case=CAVITY, collision=MRT, les=True, cs=0.12, tau=0.51,
                       u=0.1, steps=40, geometry=[("walls",)], init=("uniform", 1.0, 0.0, 0.0)),
    "cylinder_mei": dict(nx=96, ny=40, case=CYLINDER, collision=MRT, tau=0.56, u=0.1, steps=60,
                         geometry=[("cylinder", 24, 21, 4)], init=("wake", 0.1, 24, 42, 1e-4)),
    "cylinder_bgk_force": dict(nx=64, ny=32, case=CYLINDER, collision=BGK, tau=0.6, u=0.08,
                               steps=40, body_force=2e-6, geometry=[("cylinder", 16, 16, 4)],
                               init=("uniform", 1.0, 0.08, 0.0)),
    "step": dict(nx=72, ny=30, case=STEP, collision=MRT, tau=0.6, u=0.1, steps=60,
                 geometry=[("mask", "step")], init=("uniform", 1.0, 0.0, 0.0)),
    "ribs_les": dict(nx=64, ny=40, case=RIBS, collision=MRT, les=True, cs=0.1, tau=0.515, u=0.1,
                     steps=40, body_force=4e-5, geometry=[("mask", "channel3")],
                     init=("uniform", 1.0, 0.05, 0.0)),
    "hills": dict(nx=60, ny=30, case=PERIODIC_HILLS, collision=MRT, tau=0.56, u=0.1, steps=50,
                  body_force=1e-5, geometry=[("mask", "hills")], init=("uniform", 1.0, 0.1, 0.0)),
    "thermal_cavity": dict(nx=32, ny=32, case=CYLINDER, collision=MRT, tau=0.8, u=0.0, steps=60,
                           geometry=[("mask", "box")], init=("uniform", 1.0, 0.0, 0.0),
                           thermal=dict(T_ref=1.0, alpha=0.1 / 0.71, omega_k=1.0 / (0.5 + 3.0 * 0.1 / 0.71),
                                        beta=0.001, g_buoyancy=-2.0, T_init=1.0,
                                        pre=("box_walls", 1.5, 0.5), hook=(1, 1.5, 0.5))),
    "heated_cylinder": dict(nx=80, ny=36, case=CYLINDER, collision=MRT, tau=0.58, u=0.1, steps=50,
                            geometry=[("cylinder", 20, 18, 4)], init=("uniform", 1.0, 0.1, 0.0),
                            thermal=dict(T_ref=1.0, alpha=(0.08 / 3.0) / 0.71,
                                         omega_k=1.0 / (0.5 + 3.0 * (0.08 / 3.0) / 0.71),
                                         beta=0.001, g_buoyancy=-1e-3, T_init=1.0,
                                         pre=("solid_iso", 1.5), hook=(2, 1.5, 0.0))),
    "rotating_cylinder": dict(nx=80, ny=36, case=ROTATING_CYLINDER, collision=MRT, tau=0.6, u=0.1,
                              steps=50, geometry=[("cylinder", 20, 18, 4)],
                              moving_wall=(0.1 * 1.0 / 4, 20.0, 18.0),
                              init=("wake", 0.1, 20, 42, 1e-4)),
    "naca_polygon": dict(nx=96, ny=40, case=FLAT_PLATE, collision=MRT, tau=0.6, u=0.08, steps=40,
                         geometry=[("naca", 2412, 40, 30.0, 20.0, 36.0, 8.0)],
                         init=("uniform", 1.0, 0.08, 0.0)),
    "square_polygon": dict(nx=72, ny=36, case=SQUARE_CYLINDER, collision=MRT, tau=0.6, u=0.1,
                           steps=40, geometry=[("polygon", square_poly(18.3, 18.1, 4.2))],
                           init=("uniform", 1.0, 0.1, 0.0)),
    "cyl_near_wall": dict(nx=80, ny=32, case=CYLINDER_NEAR_WALL, collision=MRT, tau=0.6, u=0.1,
                          steps=40, geometry=[("cylinder", 20, 9, 4), ("row", 0)],
                          init=("uniform", 1.0, 0.1, 0.0)),
    "side_by_side": dict(nx=80, ny=40, case=SIDE_BY_SIDE, collision=MRT, tau=0.6, u=0.1, steps=40,
                         geometry=[("cylinder", 20, 12, 4), ("cylinder", 20, 28, 4)],
                         init=("wake", 0.1, 20, 7, 1e-3)),
    "cavity_cylinder_mei": dict(nx=40, ny=40, case=CAVITY, collision=MRT, tau=0.7, u=0.1, steps=40,
                                geometry=[("walls",), ("cylinder", 20, 18, 5)],
                                init=("uniform", 1.0, 0.0, 0.0)),
    "classic_bouzidi": dict(nx=64, ny=32, case=CYLINDER, collision=MRT, tau=0.6, u=0.1, steps=40,
                            geometry=[("cylinder", 16, 16, 5)], mei=False,
                            init=("uniform", 1.0, 0.1, 0.0)),
}


def named_mask(name, nx, ny):
    if name == "step":
        return step_mask(nx, ny)
    if name == "hills":
        return hills_mask(nx, ny)
    if name == "channel3":
        return channel_circles_mask(nx, ny, 3, 3, 5, seed=11)[0]
    if name == "box":
        m = np.zeros((ny, nx), np.uint8)
        m[:, 0] = 1
        m[:, nx - 1] = 1
        m[0, :] = 1
        m[ny - 1, :] = 1
        return m.reshape(-1)
    raise KeyError(name)


def polygon_of(op, naca_fn, transform_fn):
    if op[0] == "polygon":
        return np.asarray(op[1], np.float64)
    _, series, npts, cx, cy, scale, angle = op
    p = naca_fn(series, npts)
    return transform_fn(p, cx, cy, scale, angle)


def apply_setup(s, spec, naca_fn=None, transform_fn=None):
    """Drive a solver through the case's setup in driver order."""
    s.set_case(spec["case"], spec.get("collision", MRT), spec.get("les", False), spec.get("cs", 0.12))
    for op in spec["geometry"]:
        if op[0] == "walls":
            s.place_walls()
        elif op[0] == "cylinder":
            s.place_cylinder(*op[1:])
        elif op[0] in ("polygon", "naca"):
            s.place_polygon(polygon_of(op, naca_fn, transform_fn))
        elif op[0] == "row":
            ob = s.obstacle
            ob[op[1] * spec["nx"]: (op[1] + 1) * spec["nx"]] = 1
        elif op[0] == "mask":
            ob = s.obstacle
            ob[:] = np.maximum(ob, named_mask(op[1], spec["nx"], spec["ny"]))
        else:
            raise KeyError(op[0])
    if "moving_wall" in spec:
        s.set_moving_wall(True, *spec["moving_wall"])
    if not spec.get("mei", True):
        s.set_mei(False)
    if spec.get("body_force"):
        s.set_body_force(spec["body_force"])
    init = spec["init"]
    if init[0] == "uniform":
        s.init_uniform(*init[1:])
    else:
        s.init_cylinder_wake(*init[1:])
    th = spec.get("thermal")
    if th:
        s.set_thermal(True, th["T_ref"], th["alpha"], th["omega_k"], th["beta"], th["g_buoyancy"])
        s.init_thermal_uniform(th["T_init"], 0.0, 0.0)
        pre = th.get("pre")
        if pre:
            thermal_pre(s, spec, pre)


def thermal_pre(s, spec, pre):
    """The drivers' one-off thermal set-up before the loop:
    box_walls: src/thermal_cavity.cpp:107-124 (hot x=0, cold x=NX-1, adiabatic
    copy elsewhere on the wall ring); solid_iso: src/heated_cylinder.cpp:121-131."""
    nx, ny = spec["nx"], spec["ny"]
    g = s.g
    ob = s.obstacle
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    bb = [0, 3, 4, 1, 2, 7, 8, 5, 6]
    if pre[0] == "box_walls":
        Th, Tc = pre[1], pre[2]
        for y in range(ny):
            for x in range(nx):
                n = y * nx + x
                if not ob[n]:
                    continue
                if x == 0 or x == nx - 1:
                    T = Th if x == 0 else Tc
                    g[n * 9:(n + 1) * 9] = w * T * 1.0
                else:
                    gn = g[n * 9:(n + 1) * 9]
                    for i in range(9):
                        gn[i] = gn[bb[i]]
    elif pre[0] == "solid_iso":
        Tw = pre[1]
        for n in np.nonzero(ob)[0]:
            g[n * 9:(n + 1) * 9] = w * Tw * 1.0


# --------------------------------------------------------------------------- immersed boundary

# Airfoil with immersed-boundary direct forcing, set up as src/airfoil_ibm.cpp
# does: NACA polygon (naca_coords(series, npts)) centred at (NX/4, NY/2),
# chord NY/3, rotated by the angle of attack; obstacle = nodes inside the
# polygon (point_in_polygon, no bounce-back geometry); uniform equilibrium at
# u_in (cos a, sin a); Lagrangian points every `spacing` cells; tau from
# nu = u (NY/5) / Re; the default case type (CYLINDER: Zou/He inlet, outflow).
IBM_CASES = {
    "airfoil_ibm": dict(nx=120, ny=48, naca=2412, npts=100, aoa=8.0, re=100.0, u=0.1, steps=40,
                        spacing=1.5, les=False),
    "airfoil_ibm_les": dict(nx=96, ny=40, naca=12, npts=60, aoa=4.0, re=300.0, u=0.1, steps=30,
                            spacing=1.5, les=True, cs=0.12),
}


def ibm_tau(spec):
    nu = spec["u"] * (spec["ny"] / 5.0) / spec["re"]
    return 0.5 + 3.0 * nu


def ibm_setup(s, spec, naca_fn, transform_fn, pip_fn, eq_fn):
    """Drive a solver with the oracle's surface through the airfoil set-up;
    returns the airfoil polygon (the Lagrangian points are made from it)."""
    nx, ny = spec["nx"], spec["ny"]
    s.set_case(CYLINDER, MRT, spec.get("les", False), spec.get("cs", 0.12))
    poly = transform_fn(naca_fn(spec["naca"], spec["npts"]), nx / 4, ny / 2, ny / 3.0, spec["aoa"])
    ob = s.obstacle
    for y in range(ny):
        for x in range(nx):
            if pip_fn(float(x), float(y), poly):
                ob[y * nx + x] = 1
    a = spec["aoa"] * math.pi / 180.0
    eq = np.array([eq_fn(i, 1.0, spec["u"] * math.cos(a), spec["u"] * math.sin(a)) for i in range(9)])
    s.f[:] = np.tile(eq, nx * ny)
    return poly
