"""Generate the full-length golden fixtures from the reference solver itself.

Two runs at the sizes and lengths the reference's own set-ups use:

* cavity 800x300 (lid-driven cavity, MRT, tau 0.68, lid u 0.1, walls from
  place_walls, rest equilibrium), 20000 steps.  The reference's cavity
  driver forces a square grid (src/cavity.cpp:61), so the harness calls the
  solver headers directly.  Saved: the mask, the velocity on every 4th node
  in x and y, the full vertical (x = NX/2) and horizontal (y = NY/2) centre
  lines, and the total mass and kinetic energy every 1000 steps.
* cylinder wake 800x300 (src/main.cpp:51-128 at Re 100: circle R = NY/10 =
  30 at (NX/4, NY/2+1) = (200, 151), tau 0.68, u 0.1, the driver's mt19937(42)
  +-1e-4 transverse perturbation on x in [cx+5, cx+60)), 100000 steps.
  Saved: the mask, the SHA-256 of the initial populations, the per-step
  drag/lift sums for the first 4000 steps and every 10th step after that,
  and the statistics of the driver's Cd/Cl
  series computed by the reference's scripts/extract_forces.py (mean Cd,
  mean and std of Cl after the first 20%, Strouhal frequency by upward mean
  crossings after the first 40%).

Both runs go through ``oracle/_ref/libref.so`` (the unmodified reference
headers, ``make -C oracle ref``).  The cylinder run takes about 12 minutes
on 8 cores.

Usage:
    make -C oracle ref REF_SRC=<lbm-2d>/src
    python tests/golden/make_long_golden.py <lbm-2d>/scripts [cavity|cylinder]
"""
from __future__ import annotations

import hashlib
import importlib.util
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import oracle as O  # noqa: E402
import cases as CS  # noqa: E402

CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], np.float64)
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1], np.float64)

CAVITY_LONG = dict(nx=800, ny=300, tau=0.68, u=0.1, steps=20000, every=1000, stride=4)
CYLINDER_LONG = dict(nx=800, ny=300, tau=0.68, u=0.1, steps=100000, cx=200, cy=151, r=30,
                     seed=42, amp=1e-4, head=4000, dec=10, D=60.0, sat=40000)


def drag_lift(sums, c):
    """Cd, Cl of drag/lift sums as the cylinder driver normalises them (src/main.cpp:112-115)."""
    scale = 2.0 / (c["D"] * c["u"] * c["u"])
    return sums[:, 0] * scale, sums[:, 1] * scale


def onset_step(cl_dec, c, level=0.1):
    """First step (of a series sampled every c["dec"] steps) at which |Cl|
    reaches `level`: the onset of vortex shedding."""
    hit = np.nonzero(np.abs(cl_dec) >= level)[0]
    return int(hit[0]) * c["dec"] if len(hit) else -1


def macros(f):
    f = f.reshape(-1, 9)
    rho = f.sum(1)
    with np.errstate(invalid="ignore", divide="ignore"):
        return rho, (f @ CX) / rho, (f @ CY) / rho


def cavity(kind="ref"):
    c = CAVITY_LONG
    nx, ny = c["nx"], c["ny"]
    s = O.Solver(nx, ny, kind)
    s.set_case(CS.CAVITY, CS.MRT)
    s.place_walls()
    s.init_uniform(1.0, 0.0, 0.0)
    mass, ke = [], []
    t0 = time.time()
    for k in range(c["steps"] // c["every"]):
        s.step(c["tau"], c["u"], n=c["every"])
        rho, u, v = macros(s.f)
        fl = s.obstacle == 0
        mass.append(float(s.f.sum()))
        ke.append(float(0.5 * np.sum(rho[fl] * (u[fl] ** 2 + v[fl] ** 2))))
        print(f"cavity step {(k + 1) * c['every']}: mass {mass[-1]:.12e} ke {ke[-1]:.6e} "
              f"({time.time() - t0:.0f} s)", flush=True)
    rho, u, v = macros(s.f)
    U, V = u.reshape(ny, nx), v.reshape(ny, nx)
    st = c["stride"]
    out = dict(mask=s.obstacle.copy(), u_sub=U[::st, ::st].copy(), v_sub=V[::st, ::st].copy(),
               u_vcenter=U[:, nx // 2].copy(), v_vcenter=V[:, nx // 2].copy(),
               u_hcenter=U[ny // 2, :].copy(), v_hcenter=V[ny // 2, :].copy(),
               mass=np.array(mass), ke=np.array(ke), mass0=float(nx * ny))
    s.close()
    return out


def script_stats(scripts_dir, cd, cl):
    """Statistics of the driver's Cd/Cl series by the reference's own script."""
    spec = importlib.util.spec_from_file_location("extract_forces", os.path.join(scripts_dir, "extract_forces.py"))
    ef = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ef)
    steps = np.arange(len(cd), dtype=np.float64)
    n_skip = int(len(cd) * 0.2)  # scripts/extract_forces.py main(): first 20% is transient
    if n_skip < 10:
        n_skip = 0
    freq = ef.compute_strouhal(steps, cl)
    return dict(cd_mean=float(np.mean(cd[n_skip:])), cl_mean=float(np.mean(cl[n_skip:])),
                cl_std=float(np.std(cl[n_skip:])), freq=float(freq) if freq else float("nan"))


def cylinder(scripts_dir, kind="ref"):
    c = CYLINDER_LONG
    nx, ny = c["nx"], c["ny"]
    s = O.Solver(nx, ny, kind)
    s.set_case(CS.CYLINDER, CS.MRT)
    s.place_cylinder(c["cx"], c["cy"], c["r"])
    s.init_cylinder_wake(c["u"], c["cx"], c["seed"], c["amp"])
    f0_sha = hashlib.sha256(s.f.tobytes()).hexdigest()
    sums = np.zeros((c["steps"], 2))
    t0 = time.time()
    for k in range(c["steps"]):
        s.step(c["tau"], c["u"])
        sums[k] = s.force_sums()
        if (k + 1) % 5000 == 0:
            print(f"cylinder step {k + 1}: F = {sums[k]} ({time.time() - t0:.0f} s)", flush=True)
    stats = script_stats(scripts_dir, *drag_lift(sums, c))
    print("cylinder stats", stats, "St =", stats["freq"] * c["D"] / c["u"])
    out = dict(mask=s.obstacle.copy(), sums_head=sums[:c["head"]].copy(), sums_dec=sums[::c["dec"]].copy(),
               f0_sha=f0_sha, **{k: np.float64(v) for k, v in stats.items()})
    s.close()
    return out


def main():
    if not os.path.exists(O.LIB_REF):
        sys.exit("oracle/_ref/libref.so missing: build it with `make -C oracle ref`")
    if len(sys.argv) < 2:
        sys.exit(__doc__)
    which = sys.argv[2:] or ["cavity", "cylinder"]
    if "cavity" in which:
        np.savez_compressed(os.path.join(HERE, "long_cavity_800x300.npz"), **cavity())
    if "cylinder" in which:
        np.savez_compressed(os.path.join(HERE, "long_cylinder_800x300.npz"), **cylinder(sys.argv[1]))


if __name__ == "__main__":
    main()
