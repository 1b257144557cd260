"""Full-length parity at the reference's own set-ups, through the C-ABI.

The fixtures come from the reference solver itself
(tests/golden/make_long_golden.py):

* lid-driven cavity 800x300, MRT, tau 0.68, lid u 0.1, 20000 steps: the
  velocity on every 4th node, both centre lines, and the total mass and
  kinetic energy every 1000 steps.  The flow is laminar and still developing
  at 20000 steps (its kinetic energy still grows), and the fields are
  compared directly:
    - FP64 storage: velocity within 1e-9 relative L2, mass within 1e-12;
    - FP32 storage: velocity within 5e-4 relative L2, mass within 2e-6.
      The 1e-5 bound of the short golden runs does not carry over to 20000
      steps.  The flow damps a perturbation of its state (an FP64 run
      started from a state perturbed by 1e-8 ends 2e-10 from the unperturbed
      one), but it integrates the rounding of every step: the distance to
      the reference grows with steps x unit roundoff, 8e-13 for FP64
      (roundoff 1.1e-16) and 2.1e-4 for FP32 (6e-8), with the same ratio
      (about 0.4 x steps x roundoff).  Computing the boundary nodes in FP64
      or refining 1/rho by a Newton step left the FP32 figure unchanged;
    - FP16 storage (shifted deviations): velocity within 1e-3 relative L2
      against the FP64 reference, the precision bound for 16-bit storage,
      mass within 5e-6; BF16: velocity within 1e-2, mass within 2e-5.
* cylinder wake 800x300 (the Re 100 cylinder driver: R 30 at (200, 151),
  tau 0.68, u 0.1, the driver's seeded perturbation), 100000 steps.  The
  first 4000 steps of the drag/lift sums are compared as a series.  Vortex
  shedding sets in near step 37000 in the reference and saturates after
  step 50000; a storage's rounding noise seeds the instability earlier
  (FP16 by about 9000 steps, BF16 by about 18000), and the statistics of
  scripts/extract_forces.py (mean Cd and std of Cl over the last 80%,
  frequency from upward mean crossings over the last 60%) then mix in the
  growth phase.  So the saturated shedding is compared as well: mean Cd and
  std of Cl over the last 40000 steps (every 10th step).
    - FP64: everything within 1e-9 relative, the same crossing count and
      onset step;
    - FP32: series within 5e-5; the script's mean Cd within 1e-3 and Cl std
      within 2e-3; saturated mean Cd within 1e-3 and Cl std within 5e-4;
      crossing count within 1, onset within 500 steps;
    - FP16: series within 3e-3; saturated mean Cd within 5e-3 (the drag
      bound of 16-bit storage) and Cl std within 5e-3; crossing count within
      1; the script's mean Cd within 2e-2;
    - BF16: series within 2e-2; saturated mean Cd within 5e-3 and Cl std
      within 2e-2 (its lift carries visible rounding noise, which also adds
      mean crossings, so the frequency is not compared).
"""
import hashlib
import os

import numpy as np
import pytest

import cases as CS
import make_long_golden as LG
from gpu_cases import rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.dirname(os.path.abspath(CS.__file__))

CAVITY_TOL = {"fp64": (1e-9, 1e-12), "fp32": (5e-4, 2e-6), "fp16": (1e-3, 5e-6), "bf16": (1e-2, 2e-5)}
# series, script mean Cd, script Cl std, saturated mean Cd, saturated Cl std,
# crossing-count difference, onset difference in steps (None: not compared)
CYLINDER_TOL = {
    "fp64": (1e-9, 1e-9, 1e-9, 1e-9, 1e-9, 0, 0),
    "fp32": (5e-5, 1e-3, 2e-3, 1e-3, 5e-4, 1, 500),
    "fp16": (3e-3, 2e-2, None, 5e-3, 5e-3, 1, None),
    "bf16": (2e-2, None, None, 5e-3, 2e-2, None, None),
}


def cavity_metrics(product, storage):
    """Run the 20000-step cavity on the GPU and compare it with the fixture."""
    c = LG.CAVITY_LONG
    nx, ny = c["nx"], c["ny"]
    gold = np.load(os.path.join(GOLD, "long_cavity_800x300.npz"))
    g = product.Solver(nx, ny, CS.CAVITY, CS.MRT, False, 0.12, storage)
    g.place_walls()
    assert np.array_equal(g.obstacle, gold["mask"])
    g.init_uniform(1.0, 0.0, 0.0)
    fl = g.obstacle == 0
    mass, ke = [], []
    for _ in range(c["steps"] // c["every"]):
        g.step(c["tau"], c["u"], c["every"])
        f = g.f
        rho, u, v = LG.macros(f)
        mass.append(float(f.sum()))
        ke.append(float(0.5 * np.sum(rho[fl] * (u[fl] ** 2 + v[fl] ** 2))))
    g.close()
    U, V = u.reshape(ny, nx), v.reshape(ny, nx)
    st = c["stride"]
    sub = np.stack([U[::st, ::st], V[::st, ::st]])
    ref = np.stack([gold["u_sub"], gold["v_sub"]])
    m = gold["mask"].reshape(ny, nx)[::st, ::st] == 0
    lines = np.concatenate([U[:, nx // 2], V[:, nx // 2], U[ny // 2, :], V[ny // 2, :]])
    ref_lines = np.concatenate([gold["u_vcenter"], gold["v_vcenter"], gold["u_hcenter"], gold["v_hcenter"]])
    lm = np.concatenate([fl.reshape(ny, nx)[:, nx // 2]] * 2 + [fl.reshape(ny, nx)[ny // 2, :]] * 2)
    return dict(velocity=rel_l2(sub[:, m], ref[:, m]), lines=rel_l2(lines[lm], ref_lines[lm]),
                mass=float(np.max(np.abs(np.array(mass) - gold["mass"]) / gold["mass"])),
                ke=rel_l2(ke, gold["ke"]))


def cylinder_metrics(product, O, storage):
    """Run the 100000-step cylinder wake on the GPU and compare it with the fixture."""
    c = LG.CYLINDER_LONG
    nx, ny = c["nx"], c["ny"]
    gold = np.load(os.path.join(GOLD, "long_cylinder_800x300.npz"))
    s = O.Solver(nx, ny)  # the driver's initial state, from the oracle
    s.set_case(CS.CYLINDER, CS.MRT)
    s.place_cylinder(c["cx"], c["cy"], c["r"])
    s.init_cylinder_wake(c["u"], c["cx"], c["seed"], c["amp"])
    f0 = s.f.copy()
    s.close()
    assert hashlib.sha256(f0.tobytes()).hexdigest() == str(gold["f0_sha"])
    g = product.Solver(nx, ny, CS.CYLINDER, CS.MRT, False, 0.12, storage)
    g.place_cylinder(c["cx"], c["cy"], c["r"])
    assert np.array_equal(g.obstacle, gold["mask"])
    g.upload_f(f0)
    g.step(c["tau"], c["u"], c["steps"])
    fx, fy = g.force_history()
    g.close()
    assert len(fx) == c["steps"]
    sums = np.stack([fx, fy], 1)
    cd, cl = product.drag_lift_coefficients(fx, fy, c["D"], c["u"])
    st = product.force_stats(cd, cl)
    head = c["head"]
    # the frequency is (upward mean crossings) / (2 x window) over the last 60%
    window = c["steps"] - max(int(c["steps"] * 0.4), 50)
    # saturated shedding: every 10th step of the last 40000
    dec = c["dec"]
    k0 = (c["steps"] - c["sat"]) // dec
    cd_d, cl_d = cd[::dec][k0:], cl[::dec][k0:]
    rcd, rcl = LG.drag_lift(gold["sums_dec"][k0:], c)
    return dict(series=rel_l2(sums[:head], gold["sums_head"]),
                cd_mean=abs(st["mean_v1"] / float(gold["cd_mean"]) - 1.0),
                cl_std=abs(st["std_v2"] / float(gold["cl_std"]) - 1.0),
                crossings=abs(round(st["st"] * 2 * window) - round(float(gold["freq"]) * 2 * window)),
                sat_cd_mean=abs(cd_d.mean() / rcd.mean() - 1.0),
                sat_cl_std=abs(cl_d.std() / rcl.std() - 1.0),
                onset=LG.onset_step(cl[::dec], c) - LG.onset_step(rcl_all(gold, c), c),
                values=dict(cd_mean=st["mean_v1"], cl_std=st["std_v2"], freq=st["st"],
                            ref_cd_mean=float(gold["cd_mean"]), ref_cl_std=float(gold["cl_std"]),
                            ref_freq=float(gold["freq"]), sat_cd_mean=float(cd_d.mean()),
                            sat_cl_std=float(cl_d.std()), ref_sat_cd_mean=float(rcd.mean()),
                            ref_sat_cl_std=float(rcl.std())))


def rcl_all(gold, c):
    return LG.drag_lift(gold["sums_dec"], c)[1]


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16", "bf16"])
def test_cavity_800x300_20k_steps(product, storage):
    tv, tm = CAVITY_TOL[storage]
    m = cavity_metrics(product, storage)
    assert m["velocity"] < tv, m
    assert m["lines"] < tv, m
    assert m["mass"] < tm, m


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16", "bf16"])
def test_cylinder_800x300_100k_steps(product, oracle_lib, storage):
    tol = dict(zip(("series", "cd_mean", "cl_std", "sat_cd_mean", "sat_cl_std", "crossings", "onset"),
                   CYLINDER_TOL[storage]))
    m = cylinder_metrics(product, oracle_lib, storage)
    for k, t in tol.items():
        if t is not None:
            assert abs(m[k]) <= t, (k, m)
