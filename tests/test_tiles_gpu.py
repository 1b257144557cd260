"""GPU parity of the tile-pipelined step kernel (flat tiles of 512
consecutive nodes, any grid width, the thermal DDF, batches).

* Odd and unaligned widths, grids narrower than a tile (tiles span rows) and
  odd node counts (odd plane strides, split pair stores): FP32 populations
  and the drag/lift series within 1e-5 relative L2 of the oracle;
  populations within 1e-6 of the paired / one-node kernels (same arithmetic,
  separately compiled), the drag/lift series within 1e-6 of the paired
  kernel (the same FP32 grouping of a node pair's link terms) and 1e-5 of
  the one-node kernel; FP16 within the shifted-storage bound.
* The thermal DDF: against the one-node kernel (the same per-node collision
  and rounding noise) within 1e-6 (FP32) and 1e-4 (FP16).
* Batches of tile-kernel members (variant 3): every member of a mixed batch
  (odd sizes, thermal and not, FP32 and FP16) ends with the populations of
  the same solve stepped alone by the single-instance tile kernel, bit for bit (the same per-node arithmetic);
  drag/lift within 1e-12 (the second stage sums the same FP64 partials in
  another fixed order).
"""
import copy

import numpy as np
import pytest

import cases as CS
from gpu_cases import fluid_pop_mask, gpu_solver, oracle_setup, rel_l2

pytestmark = pytest.mark.gpu

ODD = {
    "ribs_les_1031x21": ("ribs_les", 1031, 21, 10),
    "ribs_les_97x33": ("ribs_les", 97, 33, 12),
    "cavity_mrt_517x13": ("cavity_mrt", 517, 13, 10),
    "step_333x30": ("step", 333, 30, 12),
    "cylinder_mei_777x41": ("cylinder_mei", 777, 41, 10),
    "cylinder_bgk_force_130x33": ("cylinder_bgk_force", 130, 33, 12),
}


def spec_of(key):
    base, nx, ny, steps = ODD[key]
    s = copy.deepcopy(CS.CASES[base])
    s["nx"], s["ny"], s["steps"] = nx, ny, steps
    if base.startswith("cylinder"):  # keep the cylinder inside the channel
        s["geometry"] = [("cylinder", nx // 4, ny // 2, ny // 5)]
    return s


def run_gpu(product, O, spec, variant, storage="fp32"):
    g = gpu_solver(product, O, spec, storage)
    g.set_kernel_variant(variant)
    kernel = g.info().kernel
    sums = []
    for _ in range(spec["steps"]):
        g.step(spec["tau"], spec["u"])
        sums.append(g.force_sums())
    f = g.f
    gg = g.g if spec.get("thermal") else None
    g.synchronize()
    g.close()
    return kernel, f, np.array(sums), gg


def run_oracle(O, spec):
    s = oracle_setup(O, spec)
    sums = []
    for _ in range(spec["steps"]):
        s.step(spec["tau"], spec["u"])
        sums.append(s.force_sums())
    f, mask = s.f.copy(), s.obstacle.copy()
    s.close()
    return f, mask, np.array(sums)


@pytest.mark.parametrize("key", sorted(ODD))
def test_tiles_match_oracle(product, oracle_lib, key):
    spec = spec_of(key)
    f_ref, mask, sums_ref = run_oracle(oracle_lib, spec)
    kern, f_t, sums_t, _ = run_gpu(product, oracle_lib, spec, 3)
    assert kern == product.KERNEL_TILES
    other = 2 if spec["nx"] % 2 == 0 else 1
    _, f_o, sums_o, _ = run_gpu(product, oracle_lib, spec, other)
    fm = fluid_pop_mask(mask)
    assert rel_l2(f_t, f_ref, fm) < 1e-5
    assert rel_l2(f_t, f_o, fm) < 1e-6
    assert np.allclose(f_t[~fm], f_ref[~fm], atol=1e-6)
    if spec["case"] != CS.CAVITY:
        assert rel_l2(sums_t, sums_ref) < 1e-5
        # the paired kernel sums a node pair's link terms in FP32 as the tile
        # kernel does; the one-node kernel (odd nx) sums one node's, so the two
        # FP32 groupings round differently (within the oracle bound)
        assert rel_l2(sums_t, sums_o) < (1e-6 if other == 2 else 1e-5)


@pytest.mark.parametrize("storage,tol", [("fp16", 5e-3), ("bf16", 3e-2)])
def test_tiles_shifted_storage(product, oracle_lib, storage, tol):
    spec = spec_of("cylinder_mei_777x41")
    f_ref, mask, _ = run_oracle(oracle_lib, spec)
    kern, f_t, _, _ = run_gpu(product, oracle_lib, spec, 3, storage)
    assert kern == product.KERNEL_TILES
    assert rel_l2(f_t, f_ref, fluid_pop_mask(mask)) < tol


THERMAL = {"thermal_cavity_130x97": ("thermal_cavity", 130, 97, 15),
           "heated_cylinder_257x61": ("heated_cylinder", 257, 61, 15)}


def thermal_spec(key):
    base, nx, ny, steps = THERMAL[key]
    s = copy.deepcopy(CS.CASES[base])
    s["nx"], s["ny"], s["steps"] = nx, ny, steps
    if base == "heated_cylinder":
        s["geometry"] = [("cylinder", nx // 4, ny // 2, ny // 5)]
    return s


@pytest.mark.parametrize("storage,tol", [("fp32", 1e-6), ("fp16", 1e-4)])
@pytest.mark.parametrize("key", sorted(THERMAL))
def test_tiles_thermal_match_one_node_kernel(product, oracle_lib, key, storage, tol):
    spec = thermal_spec(key)
    kern, f_t, sums_t, g_t = run_gpu(product, oracle_lib, spec, 3, storage)
    assert kern == product.KERNEL_TILES
    k1, f_1, sums_1, g_1 = run_gpu(product, oracle_lib, spec, 1, storage)
    assert k1 == product.KERNEL_SCALAR
    assert rel_l2(f_t, f_1) < tol
    assert rel_l2(g_t, g_1) < tol
    if key.startswith("heated_cylinder"):  # (the closed cavity's net wall force is a cancellation)
        assert rel_l2(sums_t, sums_1) < max(tol, 1e-6)


MIX = [("ribs_les_97x33", "fp32"), ("cylinder_mei_777x41", "fp16"), ("step_333x30", "fp32"),
       ("cavity_mrt_517x13", "fp16"), ("cylinder_bgk_force_130x33", "bf16")]


@pytest.mark.parametrize("steps", [9, 20])
def test_batch_members_equal_single_tiles(product, oracle_lib, steps):
    specs = [(spec_of(k), st) for k, st in MIX] + [(thermal_spec(k), st) for k, st in
                                                  (("thermal_cavity_130x97", "fp32"),
                                                   ("heated_cylinder_257x61", "fp16"))]
    alone = []
    for spec, st in specs:
        s = gpu_solver(product, oracle_lib, spec, st)
        s.set_kernel_variant(3)
        s.step(spec["tau"], spec["u"], steps)
        alone.append((s.f, s.force_history()))
        s.close()
    b = product.Batch()
    mem = []
    for spec, st in specs:
        s = gpu_solver(product, oracle_lib, spec, st)
        s.set_kernel_variant(3)  # batch members run the batched tile kernel
        b.add(s, spec["tau"], spec["u"])
        mem.append(s)
    assert all(s.info().kernel == product.KERNEL_TILES for s in mem)
    b.step(steps)
    b.synchronize()
    for (spec, st), s, (fa, (ax, ay)) in zip(specs, mem, alone):
        assert np.array_equal(s.f, fa), (spec["nx"], spec["ny"], st)
        fx, fy = s.force_history()
        assert len(fx) == len(ax)
        if len(fx):
            assert rel_l2(np.stack([fx, fy]), np.stack([ax, ay])) <= 1e-12
    b.close()
    for s in mem:
        s.close()
