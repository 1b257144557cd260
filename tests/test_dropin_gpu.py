"""The C++ drop-in path on the GPU: a driver written against the reference's
header API (tests/dropin/cylinder_driver.cpp), compiled against the drop-in
headers, runs the cylinder wake and the cavity through execute_time_step and
the fx_body/fy_body mirrors; its populations and per-step force sums match
the oracle within the FP32 tolerance (1e-5 relative L2)."""
import os
import subprocess

import numpy as np
import pytest

from dropin_build import compile_dropin
from gpu_cases import rel_l2

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("case", ["cylinder", "cavity"])
def test_dropin_driver_matches_oracle(product, oracle_lib, tmp_path, case):
    O = oracle_lib
    nx, ny, steps, tau, u = 200, 80, 60, 0.6, 0.1
    exe = tmp_path / "drv"
    r = compile_dropin(os.path.join(HERE, "dropin", "cylinder_driver.cpp"), str(exe))
    assert r.returncode == 0, r.stderr[-2000:]
    s = O.Solver(nx, ny)
    if case == "cylinder":
        s.set_case(O.CYLINDER)
        s.place_cylinder(nx // 4, ny // 2 + 1, ny // 10)
        s.init_cylinder_wake(u, nx // 4, 42, 1e-4)
        code = 0
    else:
        s.set_case(O.CAVITY)
        s.place_walls()
        s.init_uniform(1.0, 0.0, 0.0)
        code = 1
    init = tmp_path / "init.bin"
    s.f.astype("<f8").tofile(init)
    sums = []
    for _ in range(steps):
        s.step(tau, u)
        sums.append(s.force_sums())
    out = tmp_path / "out.bin"
    run = subprocess.run([str(exe), str(nx), str(ny), str(steps), str(tau), str(u), str(init), str(out), str(code)],
                         capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert run.returncode == 0, run.stderr
    data = np.fromfile(out, "<f8")
    f = data[: nx * ny * 9]
    got_sums = data[nx * ny * 9:].reshape(-1, 2)
    fl = np.repeat(s.obstacle == 0, 9)
    assert rel_l2(f, s.f, fl) < 1e-5
    if case == "cylinder":
        assert rel_l2(got_sums, np.array(sums)) < 1e-5
    assert os.path.exists(tmp_path / "dropin_out" / "frames" / f"frame_{steps}.json")
    if case == "cylinder":  # forces.jsonl from the device history: Cd = 2 Fx / (D u^2)
        import json
        rows = [json.loads(line) for line in open(tmp_path / "dropin_out" / "forces.jsonl")]
        assert len(rows) == steps
        k = 2.0 / ((ny / 5.0) * u * u)
        assert abs(rows[-1]["cd"] - k * sums[-1][0]) <= 1e-5 * abs(k * sums[-1][0]) + 1e-6
    s.close()
