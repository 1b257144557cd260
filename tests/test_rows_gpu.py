"""GPU parity of the row-pipelined step kernel on grids wider than one row
tile (512 nodes): full tiles, a partial last tile, the periodic x wrap across
tile boundaries, and the outflow column in the last tile.

Each case runs the oracle (the C restatement of the reference step) and the
GPU from the same initial state; FP32 storage must match within 1e-5
relative L2 (populations over fluid nodes, and the drag/lift series), and
the row pipeline must agree with the paired-node kernel (variant 2), which
computes the same arithmetic from register pulls, within 1e-6.
"""
import copy

import numpy as np
import pytest

import cases as CS
from gpu_cases import fluid_pop_mask, gpu_solver, oracle_setup, rel_l2

pytestmark = pytest.mark.gpu

WIDE = {
    "ribs_les_1032": ("ribs_les", 1032, 24, 12),
    "ribs_les_1028": ("ribs_les", 1028, 24, 12),  # FP32 only: nx % 8 == 4
    "ribs_les_520": ("ribs_les", 520, 20, 12),
    "step_1024": ("step", 1024, 30, 12),
    "cylinder_mei_1544": ("cylinder_mei", 1544, 40, 10),
    "cavity_mrt_1032": ("cavity_mrt", 1032, 16, 10),
}


def spec_of(key):
    base, nx, ny, steps = WIDE[key]
    s = copy.deepcopy(CS.CASES[base])
    s["nx"], s["ny"], s["steps"] = nx, ny, steps
    if base == "cylinder_mei":  # keep the cylinder inside the narrow channel
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
    g.synchronize()
    g.close()
    return kernel, f, np.array(sums)


def run_oracle(O, spec):
    s = oracle_setup(O, spec)
    sums = []
    for _ in range(spec["steps"]):
        s.step(spec["tau"], spec["u"])
        sums.append(s.force_sums())
    f, mask = s.f.copy(), s.obstacle.copy()
    s.close()
    return f, mask, np.array(sums)


@pytest.mark.parametrize("key", sorted(WIDE))
def test_rows_kernel_matches_oracle(product, oracle_lib, key):
    spec = spec_of(key)
    f_ref, mask, sums_ref = run_oracle(oracle_lib, spec)
    kern, f_rows, sums_rows = run_gpu(product, oracle_lib, spec, 0)
    assert kern == product.KERNEL_ROWS
    kp, f_pair, sums_pair = run_gpu(product, oracle_lib, spec, 2)
    assert kp == product.KERNEL_PAIR
    fm = fluid_pop_mask(mask)
    assert rel_l2(f_rows, f_ref, fm) < 1e-5
    assert rel_l2(f_rows, f_pair, fm) < 1e-6
    assert np.allclose(f_rows[~fm], f_ref[~fm], atol=1e-6)
    if spec["case"] != CS.CAVITY:
        assert rel_l2(sums_rows, sums_ref) < 1e-5
        assert rel_l2(sums_rows, sums_pair) < 1e-6


@pytest.mark.parametrize("storage,tol", [("fp16", 5e-3), ("bf16", 3e-2)])
def test_rows_kernel_shifted_storage(product, oracle_lib, storage, tol):
    spec = spec_of("ribs_les_1032")
    f_ref, mask, _ = run_oracle(oracle_lib, spec)
    kern, f_rows, _ = run_gpu(product, oracle_lib, spec, 0, storage)
    assert kern == product.KERNEL_ROWS
    _, f_pair, _ = run_gpu(product, oracle_lib, spec, 2, storage)
    fm = fluid_pop_mask(mask)
    assert rel_l2(f_rows, f_ref, fm) < tol
    # same rounding noise in both kernels; an FP32 ulp of difference before
    # the stochastic rounding can still flip a stored value by one FP16 ulp
    assert rel_l2(f_rows, f_pair, fm) < tol / 5


def test_kernel_selection(product):
    """Row pipeline only where it applies; the other kernels elsewhere."""
    s = product.Solver(1032, 8, product.RIBS)
    assert s.info().kernel == product.KERNEL_ROWS
    s.set_kernel_variant(2)
    assert s.info().kernel == product.KERNEL_PAIR
    s.set_kernel_variant(1)
    assert s.info().kernel == product.KERNEL_SCALAR
    s.close()
    for nx, storage in ((1034, "fp32"), (1036, "fp16"), (1032, "fp64")):
        s = product.Solver(nx, 8, product.RIBS, storage=storage)
        assert s.info().kernel != product.KERNEL_ROWS, (nx, storage)
        s.close()
    s = product.Solver(1036, 8, product.RIBS, storage="fp32")  # 16-byte rows in FP32
    assert s.info().kernel == product.KERNEL_ROWS
    s.close()


@pytest.mark.parametrize("variant", [0, 3])
def test_pipeline_wait_timeout_reports_and_recovers(product, oracle_lib, variant):
    """The staging pipelines' bounded waits (row pipeline, tile pipeline): in
    the failure-path test mode the producer stages nothing -- a stage that
    never fills, the flag that nothing sets -- so every consumer wait runs
    out after 2e5 SM cycles (about 0.1 ms); the kernel ends and the next
    synchronisation reports LBM2D_ERR_TIMEOUT (7).  The context stays usable:
    with the default limit restored, a re-uploaded state steps to exactly the
    result of a fresh solver."""
    spec = CS.CASES["ribs_les"]  # 64 x 40, FP32: the row pipeline, or the tile pipeline
    s = gpu_solver(product, oracle_lib, spec, "fp32")
    s.set_kernel_variant(variant)
    assert s.info().kernel == (product.KERNEL_ROWS if variant == 0 else product.KERNEL_TILES)
    f0 = s.f
    s.set_wait_limit(-200000)
    s.step(spec["tau"], spec["u"], 1)
    with pytest.raises(product.LBMError) as ex:
        s.synchronize()
    assert ex.value.code == 7
    s.set_wait_limit(0)
    s.upload_f(f0)
    s.step(spec["tau"], spec["u"], 5)
    s.synchronize()
    ref = gpu_solver(product, oracle_lib, spec, "fp32")
    ref.set_kernel_variant(variant)
    ref.step(spec["tau"], spec["u"], 5)
    assert np.array_equal(s.f, ref.f)
    s.close()
    ref.close()
