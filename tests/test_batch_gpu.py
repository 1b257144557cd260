"""Batched solves: every member's result is the same alone and in the mix.

Instances of different sizes, cases, precisions and with/without the thermal
DDF are stepped (a) one solver at a time through lbm2d_step and (b) together
through lbm2d_batch_step (one packed launch per step per storage/thermal
group, CUDA-graph replay).  The per-node arithmetic is the same source, but
the single-instance and batched kernels are compiled separately and the
compiler may fuse multiply-adds differently in each, so results agree to
rounding: populations within 1e-6 relative L2 (FP32/FP16/BF16 storage) and
1e-13 (FP64), drag/lift histories within the same relative bounds.  Members
added and removed mid-run, and the autotuner's state restore, are covered
too."""
from gpu_cases import rel_l2

TOL = {"fp64": 1e-13, "fp32": 1e-6, "fp16": 1e-6, "bf16": 1e-6}
import numpy as np
import pytest

import cases as CS
from gpu_cases import gpu_solver

pytestmark = pytest.mark.gpu

MIX = [("cavity_mrt", "fp32"), ("cylinder_mei", "fp32"), ("step", "fp16"), ("thermal_cavity", "fp32"),
       ("ribs_les", "bf16"), ("rotating_cylinder", "fp64"), ("naca_polygon", "fp32"), ("heated_cylinder", "fp32")]


def make(product, O, name, storage):
    return gpu_solver(product, O, CS.CASES[name], storage)


@pytest.mark.parametrize("steps", [7, 20])
def test_batch_equals_alone(product, oracle_lib, steps):
    alone = {}
    for name, st in MIX:
        s = make(product, oracle_lib, name, st)
        spec = CS.CASES[name]
        s.step(spec["tau"], spec["u"], steps)
        alone[name] = (s.f, s.force_history())
        s.close()
    b = product.Batch()
    mem = {}
    for name, st in MIX:
        s = make(product, oracle_lib, name, st)
        spec = CS.CASES[name]
        b.add(s, spec["tau"], spec["u"])
        mem[name] = s
    b.step(steps)
    b.synchronize()
    for name, st in MIX:
        s = mem[name]
        f, (fx, fy) = s.f, s.force_history()
        fa, (ax, ay) = alone[name]
        assert rel_l2(f, fa) <= TOL[st], name
        assert len(fx) == len(ax) == (steps if CS.CASES[name]["case"] != CS.CAVITY else 0)
        if len(fx):
            assert rel_l2(np.stack([fx, fy]), np.stack([ax, ay])) <= max(TOL[st], 1e-12), name
    b.close()
    for s in mem.values():
        s.close()


def test_batch_membership_changes(product, oracle_lib):
    """A member added late or removed early matches the same step count alone."""
    spec_a, spec_b = CS.CASES["cylinder_mei"], CS.CASES["cavity_mrt"]
    ref_a = make(product, oracle_lib, "cylinder_mei", "fp32")
    ref_a.step(spec_a["tau"], spec_a["u"], 12)
    ref_b = make(product, oracle_lib, "cavity_mrt", "fp32")
    ref_b.step(spec_b["tau"], spec_b["u"], 5)
    a = make(product, oracle_lib, "cylinder_mei", "fp32")
    bb = make(product, oracle_lib, "cavity_mrt", "fp32")
    b = product.Batch()
    b.add(a, spec_a["tau"], spec_a["u"])
    b.step(4)
    b.add(bb, spec_b["tau"], spec_b["u"])
    b.step(5)
    b.remove(bb)
    b.step(3)
    b.synchronize()
    assert rel_l2(a.f, ref_a.f) <= TOL["fp32"]
    assert rel_l2(bb.f, ref_b.f) <= TOL["fp32"]
    for s in (a, bb, ref_a, ref_b):
        s.close()
    b.close()


def test_autotune_preserves_state(product, oracle_lib):
    spec = CS.CASES["cylinder_mei"]
    ref = make(product, oracle_lib, "cylinder_mei", "fp32")
    ref.step(spec["tau"], spec["u"], 10)
    s = make(product, oracle_lib, "cylinder_mei", "fp32")
    s.step(spec["tau"], spec["u"], 4)
    bx, by = s.autotune(spec["tau"], spec["u"], steps=3)
    assert bx * by % 32 == 0
    s.step(spec["tau"], spec["u"], 6)
    fx, _ = s.force_history()
    rfx, _ = ref.force_history()
    if s.info().kernel == ref.info().kernel:
        assert np.array_equal(s.f, ref.f)
    else:  # the row pipeline and the paired kernel: same arithmetic, separately compiled
        assert rel_l2(s.f, ref.f) < 1e-6
    # the tuned shape groups nodes into warps differently: the FP32 per-warp
    # partial sums of the force round differently
    assert len(fx) == 10 and np.allclose(fx, rfx, rtol=1e-6)
    s.close()
    ref.close()


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_member_budgets(product, oracle_lib, storage):
    """Members with different step budgets share one long batched call: each
    stops exactly at its budget (steps taken, force history length) and ends
    bit-for-bit where a batch stepped for exactly that many steps ends."""
    cases = [("cylinder_mei", 9), ("step", 16), ("naca_polygon", 3), ("ribs_les", 0), ("cavity_mrt", 25)]
    b = product.Batch()
    mem = []
    for name, budget in cases:
        spec = CS.CASES[name]
        s = make(product, oracle_lib, name, storage)
        b.add(s, spec["tau"], spec["u"])
        b.set_budget(s, budget)
        mem.append(s)
    b.step(12)  # odd / even budgets below and above the call length
    b.step(12)
    b.synchronize()
    for (name, budget), s in zip(cases, mem):
        spec = CS.CASES[name]
        assert b.budget(s) == max(budget - 24, 0)
        taken = min(budget, 24)
        assert s.info().steps_done == taken, name
        ref_b = product.Batch()
        r = make(product, oracle_lib, name, storage)
        ref_b.add(r, spec["tau"], spec["u"])
        if taken:
            ref_b.step(taken)
        ref_b.synchronize()
        assert np.array_equal(s.f, r.f), name
        fx, _ = s.force_history()
        rx, _ = r.force_history()
        assert len(fx) == len(rx) == (taken if spec["case"] != CS.CAVITY else 0), name
        assert np.array_equal(fx, rx), name
        ref_b.close()
        r.close()
    b.close()
    for s in mem:
        s.close()


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_large_member_runs_solo(product, oracle_lib, storage):
    """A member of at least 2^21 nodes that qualifies for the row pipeline is
    stepped with its own row-pipeline launches inside the batch call: it
    reports that kernel, takes exactly its budget, and ends bit-for-bit where
    the same solve stepped alone ends."""
    import copy
    big = copy.deepcopy(CS.CASES["ribs_les"])
    big["nx"], big["ny"] = 2048, 1024
    small = CS.CASES["cylinder_mei"]
    b = product.Batch()
    s_big = gpu_solver(product, oracle_lib, big, storage)
    s_small = gpu_solver(product, oracle_lib, small, storage)
    b.add(s_big, big["tau"], big["u"])
    b.add(s_small, small["tau"], small["u"])
    b.set_budget(s_big, 7)
    assert s_big.info().kernel == product.KERNEL_ROWS
    assert s_small.info().kernel != product.KERNEL_ROWS
    b.step(10)
    b.synchronize()
    assert s_big.info().steps_done == 7 and s_small.info().steps_done == 10
    alone = gpu_solver(product, oracle_lib, big, storage)
    alone.step(big["tau"], big["u"], 7)
    alone.synchronize()
    assert np.array_equal(s_big.f, alone.f)
    fx, fy = s_big.force_history()
    ax, ay = alone.force_history()
    assert len(fx) == 7 and np.array_equal(fx, ax) and np.array_equal(fy, ay)
    for s in (s_big, s_small, alone):
        s.close()
    b.close()


def test_batch_autotune_preserves_state_and_budgets(product, oracle_lib):
    """Tuning the batch's block shape steps the members and undoes it: their
    steps, budgets and states are as before, and stepping on reproduces an
    untuned batch to FP32 rounding (the restored state is re-collided by the
    prologue kernel, and the block shape groups the per-warp force
    partials)."""
    names = ["cylinder_mei", "step"]

    def batch_of():
        b = product.Batch()
        mem = []
        for n in names:
            spec = CS.CASES[n]
            s = make(product, oracle_lib, n, "fp32")
            b.add(s, spec["tau"], spec["u"])
            mem.append(s)
        b.set_budget(mem[1], 9)
        return b, mem

    ref_b, ref = batch_of()
    ref_b.step(3)
    ref_b.step(10)
    ref_b.synchronize()
    b, mem = batch_of()
    b.step(3)
    b.synchronize()
    before = [s.info().steps_done for s in mem]
    b.autotune(steps=2)
    assert [s.info().steps_done for s in mem] == before
    assert b.budget(mem[0]) == -1 and b.budget(mem[1]) == 6
    b.step(10)
    b.synchronize()
    for s, r in zip(mem, ref):
        assert s.info().steps_done == r.info().steps_done
        assert rel_l2(s.f, r.f) <= 1e-6
        fx, fy = s.force_history()
        rx, ry = r.force_history()
        assert len(fx) == len(rx) and np.allclose(fx, rx, rtol=1e-6) and np.allclose(fy, ry, rtol=1e-6)
    for x in mem + ref:
        x.close()
    b.close()
    ref_b.close()


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_odd_widths_pair_on_flat_pairs(product, oracle_lib, storage):
    """Batch members of any width are stepped by the paired kernel on flat
    node pairs (2k, 2k + 1): an odd node count splits the pair stores of the
    odd planes (they would be misaligned) and stores its last node alone.
    Each agrees with the same solve stepped alone (one node per thread, or
    row pairs) to FP32 rounding."""
    import copy
    sizes = [(97, 40), (97, 41), (64, 33)]  # odd width, even N; odd width and N; even width
    specs = []
    for nx, ny in sizes:
        sp = copy.deepcopy(CS.CASES["cylinder_mei"])
        sp["nx"], sp["ny"] = nx, ny
        sp["geometry"] = [("cylinder", nx // 4, ny // 2, max(2, ny // 10))]
        sp["init"] = ("wake", 0.1, nx // 4, 42, 1e-4)
        specs.append(sp)
    b = product.Batch()
    mem = [gpu_solver(product, oracle_lib, sp, storage) for sp in specs]
    for s, sp in zip(mem, specs):
        b.add(s, sp["tau"], sp["u"])
    kinds = [s.info().kernel for s in mem]
    assert kinds == [product.KERNEL_PAIR] * 3, kinds
    b.step(30)
    b.synchronize()
    tol = {"fp32": 1e-6, "fp16": 2e-4}[storage]  # FP16: stochastic rounding apart, see test_serve_gpu
    for s, sp in zip(mem, specs):
        a = gpu_solver(product, oracle_lib, sp, storage)
        a.step(sp["tau"], sp["u"], 30)
        a.synchronize()
        assert rel_l2(s.f, a.f) <= tol, (sp["nx"], sp["ny"])
        a.close()
    b.close()
    for s in mem:
        s.close()
