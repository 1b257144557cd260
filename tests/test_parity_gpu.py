"""GPU parity: the CUDA step (through the C-ABI) against the reference.

Every golden case is run on the GPU from the same initial state and compared
with the reference's own result (tests/golden, made by the reference solver):
  * FP64 storage: populations within 1e-11 relative L2 (same algorithm,
    different rounding order), force sums within 1e-10;
  * FP32 storage (the product's plain path): populations, velocity,
    temperature and the drag/lift series within 1e-5 relative L2;
  * FP16/BF16 shifted storage: reported bounds 5e-3 / 3e-2 on populations.
Relative L2 is taken over fluid nodes (solid nodes hold the reference's
zeros, compared exactly in FP32/FP64).  The drag/lift series is compared as a
vector series: ||F_gpu - F_ref|| / ||F_ref|| over all steps and both axes.
"""
import os

import numpy as np
import pytest

import cases as CS
from gpu_cases import fluid_pop_mask, gpu_solver, rel_l2, velocity

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

TOL = {"fp64": 1e-11, "fp32": 1e-5, "fp16": 5e-3, "bf16": 3e-2}
FORCE_TOL = {"fp64": 1e-10, "fp32": 1e-5, "fp16": 2e-2, "bf16": 1e-1}


def run(product, O, spec, storage, variant=0):
    g = gpu_solver(product, O, spec, storage)
    g.set_kernel_variant(variant)
    sums = []
    for _ in range(spec["steps"]):
        g.step(spec["tau"], spec["u"])
        sums.append(g.force_sums())
    out = dict(f=g.f, sums=np.array(sums))
    fx, fy = g.force_field()
    out["fx"], out["fy"] = fx, fy
    if spec.get("thermal"):
        out["g"] = g.g
    g.synchronize()
    hist = g.force_history()
    g.close()
    out["hist"] = np.stack(hist, 1) if len(hist[0]) else np.zeros((0, 2))
    return out


@pytest.mark.parametrize("storage,variant", [("fp64", 0), ("fp32", 0), ("fp32", 1), ("fp32", 2), ("fp32", 3)])
@pytest.mark.parametrize("name", sorted(CS.CASES))
def test_gpu_matches_reference(product, oracle_lib, name, storage, variant):
    """variant 0: the fastest kernel for the case (row pipeline where nx is a
    multiple of 4 (FP32); the tile pipeline for the thermal DDF; else paired
    nodes); 1: one node per thread; 2: paired nodes per thread (packed FP32x2)
    where nx is even; 3: the tile pipeline."""
    spec = CS.CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    got = run(product, oracle_lib, spec, storage, variant)
    fm = fluid_pop_mask(gold["mask"])
    tol = TOL[storage]
    assert rel_l2(got["f"], gold["f"], fm) < tol
    # solid nodes: the reference's post-stream zeros plus boundary-condition values
    assert rel_l2(got["f"], gold["f"], ~fm) < max(tol, 1e-12) or np.allclose(got["f"][~fm], gold["f"][~fm],
                                                                             atol=1e-6)
    u, v = velocity(got["f"])
    ur, vr = velocity(gold["f"])
    fl = gold["mask"] == 0
    err_u = rel_l2(np.stack([u[fl], v[fl]]), np.stack([ur[fl], vr[fl]]))
    assert err_u < tol, (name, storage, variant, err_u)
    if "g" in gold.files:
        assert rel_l2(got["g"], gold["g"], fm) < tol
    if spec["case"] != CS.CAVITY:
        # The drag/lift error is taken relative to max(|F_net|, 1% of the gross
        # wall force sum|per-node contribution|): closed boxes (the heated
        # cavity) have a net wall force ~1/1000 of the gross force, below what
        # FP32 populations resolve; external flows are unaffected (net > 1%).
        gross = np.abs(gold["fx"]).sum() + np.abs(gold["fy"]).sum()
        net = np.linalg.norm(gold["sums"][-1])
        scale = max(1.0, 0.01 * gross / max(net, 1e-300))
        assert rel_l2(got["sums"], gold["sums"]) < FORCE_TOL[storage] * scale
        assert rel_l2(np.stack([got["fx"], got["fy"]]), np.stack([gold["fx"], gold["fy"]])) < FORCE_TOL[storage]
        assert got["hist"].shape == gold["sums"].shape
        assert np.array_equal(got["hist"], got["sums"])


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("storage", ["fp16", "bf16"])
@pytest.mark.parametrize("name", ["cavity_mrt", "cylinder_mei", "ribs_les", "thermal_cavity", "step"])
def test_gpu_shifted_storage_bounds(product, oracle_lib, name, storage, variant):
    spec = CS.CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    got = run(product, oracle_lib, spec, storage, variant)
    fm = fluid_pop_mask(gold["mask"])
    assert rel_l2(got["f"], gold["f"], fm) < TOL[storage]


def test_mass_conservation_800x300(product):
    """src/lbm_test.cpp:158-199 on the GPU path (default 800x300 grid)."""
    nx, ny = 800, 300
    s = product.Solver(nx, ny, product.CYLINDER)
    s.place_cylinder(nx // 4, ny // 2, ny // 10)
    f0 = product.equilibrium_field(nx, ny, 1.0, 0.1, 0.0)
    s.upload_f(f0)
    fluid = np.repeat(s.obstacle == 0, 9)
    m0 = f0[fluid].sum()
    s.step(0.56, 0.1, 10)
    m1 = s.f[fluid].sum()
    s.close()
    assert abs(m1 - m0) < 0.01 * m0


def test_device_diagnostics(product, oracle_lib):
    """Mass/momentum reductions (FP64 on the device) against the oracle's
    state, and the steady-state residual shrinking as a cavity converges."""
    spec = CS.CASES["cavity_mrt"]
    s = oracle_lib.Solver(spec["nx"], spec["ny"])
    CS.apply_setup(s, spec)
    g = gpu_solver(product, oracle_lib, spec, "fp64")
    s.step(spec["tau"], spec["u"], 30)
    g.step(spec["tau"], spec["u"], 30)
    m, jx, jy, r0 = g.diagnostics()
    f = s.f.reshape(-1, 9)[s.obstacle == 0]
    cx = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
    cy = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
    assert abs(m - f.sum()) < 1e-12 * f.sum()
    assert abs(jx - (f @ cx).sum()) < 1e-11 and abs(jy - (f @ cy).sum()) < 1e-11
    assert np.isnan(r0)
    res = []
    for _ in range(4):
        g.step(spec["tau"], spec["u"], 200)
        res.append(g.diagnostics()[3])
    assert all(np.isfinite(res)) and res[-1] < res[0]
    s.close()
    g.close()


def test_parameter_change_between_steps(product, oracle_lib):
    """tau and the body force may change between execute_time_step calls; the
    stored post-collision state is re-collided so results stay exact."""
    spec = dict(CS.CASES["ribs_les"])
    s = oracle_lib.Solver(spec["nx"], spec["ny"])
    CS.apply_setup(s, spec)
    g = gpu_solver(product, oracle_lib, spec, "fp64")
    taus = [0.515, 0.53, 0.53, 0.6, 0.515]
    for k, tau in enumerate(taus):
        bf = 4e-5 if k % 2 == 0 else 1e-5
        s.set_body_force(bf)
        g.set_body_force(bf)
        s.step(tau, 0.1)
        g.step(tau, 0.1)
    assert rel_l2(g.f, s.f, fluid_pop_mask(s.obstacle)) < 1e-11
    s.close()
    g.close()


def test_mask_change_between_steps(product, oracle_lib):
    spec = CS.CASES["cylinder_mei"]
    s = oracle_lib.Solver(spec["nx"], spec["ny"])
    CS.apply_setup(s, spec)
    g = gpu_solver(product, oracle_lib, spec, "fp64")
    for k in range(6):
        if k == 3:
            s.place_cylinder(60, 20, 3)
            g.place_cylinder(60, 20, 3)
        s.step(spec["tau"], spec["u"])
        g.step(spec["tau"], spec["u"])
    assert np.array_equal(g.obstacle, s.obstacle)
    assert rel_l2(g.f, s.f, fluid_pop_mask(s.obstacle)) < 1e-11
    s.close()
    g.close()


def test_nan_is_reported(product):
    s = product.Solver(32, 32, product.CAVITY)
    s.place_walls()
    f = product.equilibrium_field(32, 32, 1.0, 0.0, 0.0)
    f[(16 * 32 + 16) * 9: (16 * 32 + 17) * 9] = np.nan
    s.upload_f(f)
    s.step(0.6, 0.1, 2)
    with pytest.raises(product.LBMError) as e:
        s.synchronize()
    assert e.value.code == 4
    s.close()


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("name", ["cylinder_mei", "cavity_les", "ribs_les", "step", "thermal_cavity"])
def test_multi_step_call_equals_single_steps(product, oracle_lib, name, storage):
    """lbm2d_step with n steps (whole step pairs replayed from a captured
    CUDA graph) gives the same bits, force history and seed sequence as n
    calls of one step (plain launches)."""
    spec = CS.CASES[name]
    a = gpu_solver(product, oracle_lib, spec, storage)
    b = gpu_solver(product, oracle_lib, spec, storage)
    n = spec["steps"]
    a.step(spec["tau"], spec["u"], n)
    for _ in range(n):
        b.step(spec["tau"], spec["u"])
    assert np.array_equal(a.f, b.f)
    ha, hb = a.force_history(), b.force_history()
    assert np.array_equal(np.stack(ha), np.stack(hb))
    a.step(spec["tau"], spec["u"], 7)  # odd count: pairs + one plain step, graph reused
    for _ in range(7):
        b.step(spec["tau"], spec["u"])
    assert np.array_equal(a.f, b.f)
    a.close()
    b.close()
