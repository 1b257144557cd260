"""Drag/lift post-processing (the reference's scripts/extract_forces.py
restated in the library) against a direct restatement in numpy on force
series produced by the oracle's cylinder wake."""
import math

import numpy as np


def _script_stats(v1, v2, dt=1.0):
    # scripts/extract_forces.py:91-121 (compute_strouhal) and :137-158 (main)
    n = len(v1)
    n_skip = int(n * 0.2)
    if n_skip < 10:
        n_skip = 0
    out = dict(mean_v1=np.mean(v1[n_skip:]), mean_v2=np.mean(v2[n_skip:]), std_v2=np.std(v2[n_skip:]))
    st = None
    if n >= 200:
        skip = max(int(n * 0.4), 50)
        seg = v2[skip:]
        if len(seg) >= 100:
            m = np.mean(seg)
            c = sum(1 for i in range(1, len(seg)) if seg[i - 1] < m and seg[i] >= m)
            if c >= 2:
                st = c / (2.0 * len(seg) * dt)
    out["st"] = st
    return out


def test_force_stats_match_script(product, oracle_lib):
    O = oracle_lib
    s = O.Solver(120, 48)
    s.set_case(O.CYLINDER)
    s.place_cylinder(30, 25, 5)
    s.init_cylinder_wake(0.1, 30, 42, 1e-3)
    fx, fy = [], []
    for _ in range(260):
        s.step(0.53, 0.1)
        a, b = s.force_sums()
        fx.append(a)
        fy.append(b)
    s.close()
    cd, cl = product.drag_lift_coefficients(fx, fy, 48 / 5.0, 0.1)
    got = product.force_stats(cd, cl)
    ref = _script_stats(cd, cl)
    for k in ("mean_v1", "mean_v2", "std_v2"):
        assert math.isclose(got[k], ref[k], rel_tol=1e-12, abs_tol=1e-15), k
    if ref["st"] is None:
        assert math.isnan(got["st"])
    else:
        assert math.isclose(got["st"], ref["st"], rel_tol=1e-12)
    # a synthetic lift with a known period
    t = np.arange(2000)
    lift = np.sin(2 * np.pi * t / 50.0 + 0.3)
    st = product.force_stats(np.ones_like(lift), lift)["st"]
    assert math.isclose(st, _script_stats(np.ones_like(lift), lift)["st"], rel_tol=1e-12)
