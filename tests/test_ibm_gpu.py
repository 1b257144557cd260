"""Immersed-boundary direct forcing on the device (lbm2d_set_ibm) against
the reference's airfoil driver loop (src/airfoil_ibm.cpp:121-176 with
src/ibm.hpp), whose results are the golden fixtures airfoil_ibm*.npz made by
the reference itself (tests/golden/make_golden.py).

Same initial state, mask and Lagrangian points; after the steps:
  * populations over fluid nodes within 1e-11 (FP64 storage) / 1e-5 (FP32)
    relative L2 (5e-3 for FP16), for every step kernel;
  * the Lagrangian velocities and forces of the last iteration and the
    per-step momentum-exchange sums within the same bounds.
"""
import os

import numpy as np
import pytest

import cases as CS
from gpu_cases import fluid_pop_mask, rel_l2

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {"fp64": 1e-11, "fp32": 1e-5, "fp16": 5e-3}


def make(product, name, storage, variant=0):
    spec = CS.IBM_CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    s = product.Solver(spec["nx"], spec["ny"], CS.CYLINDER, CS.MRT, spec["les"], spec.get("cs", 0.12), storage)
    s.set_mask(gold["mask"])
    s.upload_f(gold["f0"])
    s.set_kernel_variant(variant)
    pts = product.ibm_points_from_polygon(gold["poly"], spec["spacing"])
    s.set_ibm(pts)
    return spec, gold, s, pts


@pytest.mark.parametrize("storage,variant", [("fp64", 0), ("fp32", 0), ("fp32", 1), ("fp32", 2), ("fp16", 0)])
@pytest.mark.parametrize("name", sorted(CS.IBM_CASES))
def test_ibm_matches_reference(product, name, storage, variant):
    spec, gold, s, pts = make(product, name, storage, variant)
    assert np.array_equal(pts, gold["points"])
    tau = CS.ibm_tau(spec)
    sums = []
    for _ in range(spec["steps"]):
        s.step(tau, spec["u"])
        sums.append(s.force_sums())
    tol = TOL[storage]
    fm = fluid_pop_mask(gold["mask"])
    assert rel_l2(s.f, gold["f"], fm) < tol
    U, V, FX, FY = s.ibm_lagrangian()
    assert rel_l2(np.stack([U, V]), np.stack([gold["U"], gold["V"]])) < 10 * tol
    assert rel_l2(np.stack([FX, FY]), np.stack([gold["FX"], gold["FY"]])) < 10 * tol
    if np.any(gold["sums"]):
        assert rel_l2(np.array(sums), gold["sums"]) < 10 * tol
    s.close()


def test_ibm_one_call_equals_per_step_calls(product):
    """n steps in one lbm2d_step equal n calls of one step, and the
    no-allocation entry point gives the same bits."""
    name = "airfoil_ibm"
    spec = CS.IBM_CASES[name]
    tau = CS.ibm_tau(spec)
    _, gold, a, _ = make(product, name, "fp32")
    a.step(tau, spec["u"], spec["steps"])
    _, _, b, _ = make(product, name, "fp32")
    for _ in range(spec["steps"]):
        b.step(tau, spec["u"])
    _, _, c, _ = make(product, name, "fp32")
    c.step(tau, spec["u"], 2)
    rc = c.L.lbm2d_step_noalloc(c.h, tau, spec["u"], spec["steps"] - 2)
    assert rc == 0
    fa, fb, fc = a.f, b.f, c.f
    assert np.array_equal(fa, fb) and np.array_equal(fa, fc)
    for s in (a, b, c):
        s.close()


def test_ibm_parameter_change_and_removal(product):
    """A tau change mid-run re-collides the forced state (no jump in the
    forcing); removing the boundary leaves plain steps."""
    name = "airfoil_ibm"
    spec = CS.IBM_CASES[name]
    tau = CS.ibm_tau(spec)
    _, gold, a, pts = make(product, name, "fp64")
    _, _, b, _ = make(product, name, "fp64")
    a.step(tau, spec["u"], 10)
    b.step(tau, spec["u"], 10)
    a.step(tau * 1.01, spec["u"], 5)
    b.f  # round trip through the staged state
    b.upload_f(b.f)
    b.step(tau * 1.01, spec["u"], 5)
    assert rel_l2(a.f, b.f) < 1e-13
    a.set_ibm(np.zeros((0, 2)))
    a.step(tau, spec["u"], 3)
    assert np.isfinite(a.f).all()
    with pytest.raises(product.LBMError):
        a.ibm_lagrangian()
    a.close()
    b.close()


def test_ibm_rejected_with_thermal_and_in_batch(product):
    name = "airfoil_ibm"
    _, _, s, pts = make(product, name, "fp32")
    with pytest.raises(product.LBMError):
        s.set_thermal(True, 1.0, 0.02, 1.0, 0.001, 0.5)
    b = product.Batch()
    with pytest.raises(product.LBMError):
        b.add(s, 0.6, 0.1)
    b.close()
    s.close()


@pytest.mark.parametrize("name", sorted(CS.IBM_CASES))
def test_dropin_ibm_driver_matches_reference(product, tmp_path, name):
    """A driver on the drop-in headers (ImmersedBoundary + attach_ibm, then
    execute_time_step alone) reproduces the reference's airfoil loop."""
    import subprocess

    from dropin_build import compile_dropin
    spec = CS.IBM_CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    exe = tmp_path / "ibm_drv"
    here = os.path.dirname(os.path.abspath(__file__))
    r = compile_dropin(os.path.join(here, "dropin", "ibm_driver.cpp"), str(exe))
    assert r.returncode == 0, r.stderr[-2000:]
    out = tmp_path / "out.bin"
    args = [spec["nx"], spec["ny"], spec["steps"], repr(CS.ibm_tau(spec)), spec["u"], spec["naca"], spec["npts"],
            spec["aoa"], spec["spacing"], int(spec["les"]), out]
    run = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stderr
    data = np.fromfile(out, "<f8")
    n9 = spec["nx"] * spec["ny"] * 9
    f, lag = data[:n9], data[n9:].reshape(4, -1)
    assert rel_l2(f, gold["f"], fluid_pop_mask(gold["mask"])) < 1e-5
    assert rel_l2(lag[2:], np.stack([gold["FX"], gold["FY"]])) < 1e-4
