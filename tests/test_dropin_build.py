"""The reference's own case drivers and unit tests compile UNCHANGED against
the drop-in headers (lbm-2d_gb300/dropin) and link liblbm2d; the unit tests
that need no GPU run.  Each source is copied to a temporary directory so its
quoted includes resolve to the drop-in headers, not to the reference's own.
Skipped unless LBM2D_REF_SRC names the reference's src/ folder."""
import os
import shutil
import subprocess

import pytest

from dropin_build import compile_dropin

# the reference's src/ folder, from the environment (no default)
REF_SRC = os.environ.get("LBM2D_REF_SRC", "")
DRIVERS = ["main", "cavity", "step", "thermal_cavity", "heated_cylinder", "rotating_cylinder",
           "side_by_side_cylinders", "cylinder_near_wall", "periodic_hills", "square_cylinder", "flat_plate",
           "orifice_plate", "urban_canyon", "downwash", "airfoil_ibm"]

needs_ref = pytest.mark.skipif(not (REF_SRC and os.path.isdir(REF_SRC)),
                               reason="LBM2D_REF_SRC does not name the reference sources")


@needs_ref
@pytest.mark.parametrize("name", DRIVERS)
def test_reference_driver_compiles_against_dropin(product, tmp_path, name):
    src = tmp_path / f"{name}.cpp"
    shutil.copy(os.path.join(REF_SRC, f"{name}.cpp"), src)
    r = compile_dropin(str(src), str(tmp_path / name), extra_after=REF_SRC)
    assert r.returncode == 0, r.stderr[-2000:]
    nm = subprocess.run(["nm", "-D", "--undefined-only", str(tmp_path / name)], capture_output=True, text=True)
    assert "lbm2d_step" in nm.stdout  # the step goes through the C-ABI


@needs_ref
def test_reference_unit_tests_on_dropin(product, tmp_path):
    """src/lbm_test.cpp built against the drop-in; the host-side tests run
    here (TimeStepTest needs a GPU and runs in the GPU suite's own driver)."""
    src = tmp_path / "lbm_test.cpp"
    shutil.copy(os.path.join(REF_SRC, "lbm_test.cpp"), src)
    exe = tmp_path / "lbm_test"
    r = compile_dropin(str(src), str(exe), extra_after=REF_SRC)
    assert r.returncode == 0, r.stderr[-2000:]
    env = dict(os.environ, LBM2D_TEST_SKIP="TimeStep")
    run = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=120)
    assert run.returncode == 0, run.stdout
    assert "11 tests, 0 failed" in run.stdout


def test_own_dropin_driver_compiles(product, tmp_path):
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dropin", "cylinder_driver.cpp")
    r = compile_dropin(src, str(tmp_path / "drv"))
    assert r.returncode == 0, r.stderr[-2000:]
