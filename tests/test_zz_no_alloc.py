"""lbm2d_step_noalloc: the step entry point that allocates nothing.

Callers that may not allocate device memory while they run (real-time loops
with a per-step deadline, processes whose device footprint is fixed at
start-up) prepare a solver once with lbm2d_step and then advance it with
lbm2d_step_noalloc, whose force-reduction scratch is a fixed array compiled
into the library.  This test calls it through the C-ABI twice in a row and
checks each result against the regular entry point on an identical solver:
populations within the FP32 parity bound of the other GPU tests (1e-5
relative L2) and the per-step drag/lift within the same bound.  It also
checks that the device's free memory does not change across either call:
the preparing lbm2d_step has already looked the fixed array up on the
device, and the allocation-free call launches only kernels that lbm2d_step
has loaded.  It runs last (file name) so a failure here cannot hide another
test.
"""
import ctypes as C

import numpy as np
import pytest

import cases as CS
from gpu_cases import gpu_solver, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def test_noalloc_step_matches_regular_step(product, oracle_lib):
    L = product.lib()
    fn = L.lbm2d_step_noalloc
    fn.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
    fn.restype = C.c_int
    spec = CS.CASES["cylinder_mei"]  # has momentum-exchange links, so the scratch is used
    tau, u = spec["tau"], spec["u"]
    regular = gpu_solver(product, oracle_lib, spec, "fp32")
    noalloc = gpu_solver(product, oracle_lib, spec, "fp32")
    # set-up through the regular entry point (it allocates what the solver needs)
    regular.step(tau, u, 1)
    noalloc.step(tau, u, 1)
    assert noalloc.info().n_force_nodes > 0
    for call in range(2):
        regular.step(tau, u, 6)
        free_before = _free_bytes()
        rc = fn(noalloc.h, tau, u, 6)
        assert rc == 0, L.lbm2d_last_error(noalloc.h).decode()
        noalloc.synchronize()
        assert _free_bytes() == free_before, call
        assert rel_l2(noalloc.f, regular.f) <= TOL
        fx_a, fy_a = regular.force_history()
        fx_b, fy_b = noalloc.force_history()
        assert len(fx_a) == len(fx_b) == 1 + 6 * (call + 1)
        assert rel_l2(np.stack([fx_b, fy_b]), np.stack([fx_a, fy_a])) <= TOL
        assert noalloc.force_sums() == (fx_b[-1], fy_b[-1])
    regular.close()
    noalloc.close()


def test_noalloc_step_rejects_unprepared_solver(product, oracle_lib):
    L = product.lib()
    fn = L.lbm2d_step_noalloc
    fn.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int]
    fn.restype = C.c_int
    spec = CS.CASES["cylinder_mei"]
    s = gpu_solver(product, oracle_lib, spec, "fp32")
    assert fn(s.h, spec["tau"], spec["u"], 1) == 5  # LBM2D_ERR_STATE: not prepared yet
    s.step(spec["tau"], spec["u"], 1)
    assert fn(s.h, spec["tau"] * 1.1, spec["u"], 1) == 5  # tau changed: needs the regular path
    assert fn(s.h, spec["tau"], spec["u"], 1) == 0
    s.set_profiling(True)
    assert fn(s.h, spec["tau"], spec["u"], 1) == 5  # profiling events are the regular path's
    s.set_profiling(False)
    assert fn(s.h, spec["tau"], spec["u"], 1) == 0
    s.close()
