"""The oracle (C restatement) against fixtures made by the reference itself.

Every case of tests/golden/cases.py was run through the reference solver's
own headers (tests/golden/make_golden.py); the restatement must reproduce the
mask, the final populations, the per-node force fields, the per-step force
sums and the wall distance BIT FOR BIT.
"""
import os

import numpy as np
import pytest

import cases as CS

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def run_oracle(O, spec):
    s = O.Solver(spec["nx"], spec["ny"], "oracle")
    CS.apply_setup(s, spec, naca_fn=O.naca_coords, transform_fn=O.transform_points)
    mask = s.obstacle.copy()
    th = spec.get("thermal")
    hook = th.get("hook") if th else None
    sums = []
    for _ in range(spec["steps"]):
        s.step(spec["tau"], spec["u"])
        if hook:
            s.thermal_hook(*hook)
        sums.append(s.force_sums())
    out = dict(mask=mask, f=s.f.copy(), fx=s.fx.copy(), fy=s.fy.copy(), sums=np.array(sums))
    if th:
        out["g"] = s.g.copy()
    if spec.get("les"):
        out["wall_dist"] = s.wall_dist.copy()
    s.close()
    return out


@pytest.mark.parametrize("name", sorted(CS.CASES))
def test_oracle_matches_reference_bit_exact(oracle_lib, name):
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    got = run_oracle(oracle_lib, CS.CASES[name])
    for key in gold.files:
        a, b = got[key], gold[key]
        assert a.shape == b.shape, key
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"{name}:{key} differs"


def run_oracle_ibm(O, spec):
    """The airfoil immersed-boundary loop on the restatement."""
    s = O.Solver(spec["nx"], spec["ny"], "oracle")
    poly = CS.ibm_setup(s, spec, naca_fn=O.naca_coords, transform_fn=O.transform_points,
                        pip_fn=O.point_in_polygon, eq_fn=O.equilibrium)
    out = {"mask": s.obstacle.copy(), "f0": s.f.copy(), "poly": poly}
    out["points"] = s.ibm_from_polygon(poly, spec["spacing"])
    sums = []
    for _ in range(spec["steps"]):
        s.ibm_step(CS.ibm_tau(spec), spec["u"])
        sums.append(s.force_sums())
    out["f"] = s.f.copy()
    out["U"], out["V"], out["FX"], out["FY"] = s.ibm_lagrangian()
    out["sums"] = np.array(sums)
    s.close()
    return out


@pytest.mark.parametrize("name", sorted(CS.IBM_CASES))
def test_oracle_ibm_matches_reference_bit_exact(oracle_lib, name):
    """Immersed-boundary forcing (src/ibm.hpp with the loop of
    src/airfoil_ibm.cpp:121-176): points, final populations, Lagrangian
    velocities and forces bit for bit."""
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    got = run_oracle_ibm(oracle_lib, CS.IBM_CASES[name])
    for key in gold.files:
        a, b = np.asarray(got[key]), gold[key]
        assert a.shape == b.shape, key
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"{name}:{key} differs"


def test_geometry_known_answers(oracle_lib):
    O = oracle_lib
    kat = np.load(os.path.join(GOLD, "kat.npz"))
    for series, n in ((12, 50), (2412, 60), (4415, 33)):
        assert np.array_equal(O.naca_coords(series, n), kat[f"naca_{series}_{n}"])
    p = O.transform_points(O.naca_coords(2412, 40), 30.0, 20.0, 36.0, 8.0)
    assert np.array_equal(p, kat["transform_2412"])
    pip = [O.point_in_polygon(x, y, p) for x, y in kat["pip_pts"]]
    assert np.array_equal(np.array(pip, np.uint8), kat["pip"])
    eq = [[O.equilibrium(i, rho, u, v) for i in range(9)]
          for rho, u, v in ((1.0, 0.0, 0.0), (1.2, 0.1, 0.05), (1.5, 0.12, -0.08), (0.9, -0.07, 0.11))]
    assert np.array_equal(np.array(eq), kat["equilibrium"])
    s = O.Solver(48, 40)
    s.place_cylinder(20, 21, 7)
    qs = [s.compute_q(x, y, i) for x in range(10, 31) for y in range(11, 32) for i in range(9)]
    assert np.array_equal(np.array(qs), kat["q_cylinder"])
    s.close()
    s = O.Solver(96, 40)
    s.place_polygon(p)
    qs = [s.compute_q(x, y, i) for x in range(26, 70, 2) for y in range(14, 28) for i in range(9)]
    assert np.array_equal(np.array(qs), kat["q_polygon"])
    s.close()


# Restatements of the reference's own unit tests (src/lbm_test.cpp) on the oracle.
def test_equilibrium_sums_and_momentum(oracle_lib):
    O = oracle_lib
    assert abs(sum(O.equilibrium(i, 1.2, 0.1, 0.05) for i in range(9)) - 1.2) < 1e-12
    cx = [0, 1, 0, -1, 0, 1, -1, -1, 1]
    cy = [0, 0, 1, 0, -1, 1, 1, -1, -1]
    mx = sum(O.equilibrium(i, 1.0, 0.15, 0.0) * cx[i] for i in range(9))
    my = sum(O.equilibrium(i, 1.0, 0.15, 0.0) * cy[i] for i in range(9))
    assert abs(mx - 0.15) < 1e-12 and abs(my) < 1e-12
    w = [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4
    for i in range(9):
        assert abs(O.equilibrium(i, 1.0, 0.0, 0.0) - w[i]) < 1e-15
        assert O.equilibrium(i, 1.0, 0.1, 0.05) > 0.0


def test_mass_conservation_10_steps(oracle_lib):
    """src/lbm_test.cpp:158-199 at the reference's default 800x300 grid."""
    O = oracle_lib
    s = O.Solver(800, 300)
    s.set_case(O.CYLINDER)
    s.place_cylinder(200, 150, 30)
    s.init_uniform(1.0, 0.1, 0.0)
    fluid = s.obstacle == 0
    m0 = s.f.reshape(-1, 9)[fluid].sum()
    s.step(0.56, 0.1, n=10)
    m1 = s.f.reshape(-1, 9)[fluid].sum()
    s.close()
    assert abs(m1 - m0) < 0.01 * m0


def test_oracle_long_setups_match_reference(oracle_lib):
    """The full-length fixtures (tests/golden/make_long_golden.py): the
    restatement reproduces their masks, the cylinder driver's seeded initial
    state (SHA-256 of the populations), the first 300 drag/lift sums of the
    cylinder wake and the cavity's total mass after 1000 steps, bit for bit."""
    import hashlib

    import make_long_golden as LG
    O = oracle_lib
    c = LG.CYLINDER_LONG
    gold = np.load(os.path.join(GOLD, "long_cylinder_800x300.npz"))
    s = O.Solver(c["nx"], c["ny"], "oracle")
    s.set_case(CS.CYLINDER, CS.MRT)
    s.place_cylinder(c["cx"], c["cy"], c["r"])
    s.init_cylinder_wake(c["u"], c["cx"], c["seed"], c["amp"])
    assert np.array_equal(s.obstacle, gold["mask"])
    assert hashlib.sha256(s.f.tobytes()).hexdigest() == str(gold["f0_sha"])
    sums = []
    for _ in range(300):
        s.step(c["tau"], c["u"])
        sums.append(s.force_sums())
    s.close()
    assert np.array_equal(np.array(sums), gold["sums_head"][:300])
    c = LG.CAVITY_LONG
    gold = np.load(os.path.join(GOLD, "long_cavity_800x300.npz"))
    s = O.Solver(c["nx"], c["ny"], "oracle")
    s.set_case(CS.CAVITY, CS.MRT)
    s.place_walls()
    s.init_uniform(1.0, 0.0, 0.0)
    assert np.array_equal(s.obstacle, gold["mask"])
    s.step(c["tau"], c["u"], n=c["every"])
    assert float(s.f.sum()) == float(gold["mass"][0])
    s.close()
