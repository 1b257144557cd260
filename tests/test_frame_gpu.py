"""Frame export on the device (lbm2d_frame_fields): the fields of the
reference's frame writers (src/lbm.hpp:588-701 JSON, :707-817 thermal JSON,
:860-926 VTK) computed from the device state.

* Bit-exact against a numpy restatement of the writers' arithmetic applied to
  the state the same solver downloads (lbm2d_download_f / _g): the kernel
  uses the reference's FP64 operation order with nothing fused.
* Against the reference: the same restatement on the golden cases' final
  states (made by the reference solver), within the storage's tolerance.
* The drop-in writers (tests/dropin/frame_driver.cpp) write byte-identical
  JSON / thermal JSON / VTK files from the device fields and from the host
  mirrors.
"""
import os
import subprocess

import numpy as np
import pytest

import cases as CS
from dropin_build import compile_dropin
from gpu_cases import gpu_solver, rel_l2

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
CX = (0, 1, 0, -1, 0, 1, -1, -1, 1)
CY = (0, 0, 1, 0, -1, 1, 1, -1, -1)
KEYS = ("rho", "u", "v", "vel", "omega", "T")


def writer_fields(f, g, mask, nx, ny, ds, sanitize=True, T_wall=0.0):
    """numpy restatement of the frame writers' per-point fields
    (src/lbm.hpp:609-653): compute_macros with sequential sums, u = mx/rho,
    the JSON replacements, speed, and the downsampled vorticity stencil."""
    f = f.reshape(ny, nx, 9)[::ds, ::ds]
    ob = mask.reshape(ny, nx)[::ds, ::ds] != 0
    nyd, nxd = ob.shape
    rho = np.zeros((nyd, nxd))
    mx = np.zeros((nyd, nxd))
    my = np.zeros((nyd, nxd))
    for q in range(9):
        rho = rho + f[..., q]
        mx = mx + f[..., q] * float(CX[q])
        my = my + f[..., q] * float(CY[q])
    with np.errstate(invalid="ignore", divide="ignore"):
        u = mx / rho
        v = my / rho
    T = np.zeros((nyd, nxd))
    if g is not None:
        gg = g.reshape(ny, nx, 9)[::ds, ::ds]
        for q in range(9):
            T = T + gg[..., q]
    if sanitize:
        bad = (rho < 1e-12) | np.isnan(rho)
        rho[bad], u[bad], v[bad] = 1.0, 0.0, 0.0
        u[np.isnan(u)] = 0.0
        v[np.isnan(v)] = 0.0
        if g is not None:
            T[np.isnan(T)] = 1.0
    with np.errstate(invalid="ignore"):
        vel = np.sqrt(u * u + v * v)
    if sanitize:
        vel[np.isnan(vel)] = 0.0
    for a in (rho, u, v, vel):
        a[ob] = 0.0
    T[ob] = T_wall
    I, J = np.arange(nxd), np.arange(nyd)
    il, ir = np.maximum(I - 1, 0), np.minimum(I + 1, nxd - 1)
    jd, ju = np.maximum(J - 1, 0), np.minimum(J + 1, nyd - 1)
    with np.errstate(invalid="ignore", divide="ignore"):
        dvdx = (v[:, ir] - v[:, il]) / (2.0 * ((ir - il) * ds).astype(np.float64))[None, :]
        dudy = (u[ju, :] - u[jd, :]) / (2.0 * ((ju - jd) * ds).astype(np.float64))[:, None]
    om = dvdx - dudy
    om[ob] = 0.0
    return dict(rho=rho, u=u, v=v, vel=vel, omega=om, T=T, obstacle=ob.astype(np.uint8))


def _run(product, O, name, storage, steps=None):
    spec = CS.CASES[name]
    g = gpu_solver(product, O, spec, storage)
    for _ in range(steps or spec["steps"]):
        g.step(spec["tau"], spec["u"])
    return spec, g


CASES = ["cylinder_mei", "cavity_mrt", "thermal_cavity", "heated_cylinder", "step", "ribs_les"]


@pytest.mark.parametrize("storage", ["fp64", "fp32", "fp16"])
@pytest.mark.parametrize("name", CASES)
def test_frame_fields_bit_exact(product, oracle_lib, name, storage):
    spec, g = _run(product, oracle_lib, name, storage)
    nx, ny = spec["nx"], spec["ny"]
    th = bool(spec.get("thermal"))
    f = g.f
    gg = g.g if th else None
    mask = g.obstacle
    for ds in (1, 2, 3, max(1, nx // 100)):
        for san in (True, False):
            got = g.frame_fields(ds, sanitize=san, T_wall=0.75)
            want = writer_fields(f, gg, mask, nx, ny, ds, san, 0.75)
            for k in KEYS:
                if k == "T" and not th:
                    assert np.all(got[k][want["obstacle"] == 0] == 0.0)
                    continue
                assert np.array_equal(got[k], want[k], equal_nan=True), (k, ds, san)
            assert np.array_equal(got["obstacle"], want["obstacle"])
    g.close()


@pytest.mark.parametrize("storage,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
@pytest.mark.parametrize("name", CASES)
def test_frame_fields_match_reference(product, oracle_lib, name, storage, tol):
    spec, g = _run(product, oracle_lib, name, storage)
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    nx, ny = spec["nx"], spec["ny"]
    th = bool(spec.get("thermal"))
    ds = max(1, nx // 100)
    got = g.frame_fields(ds)
    want = writer_fields(gold["f"], gold["g"] if th else None, gold["mask"], nx, ny, ds)
    fl = want["obstacle"] == 0
    assert np.array_equal(got["obstacle"], want["obstacle"])
    for k in ("rho", "u", "v", "vel") + (("T",) if th else ()):
        assert rel_l2(got[k], want[k], fl) < tol, k
    # the vorticity is a difference of neighbouring velocities: 10x the bound
    assert rel_l2(got["omega"], want["omega"], fl) < 10 * tol
    g.close()


def test_frame_fields_errors(product, oracle_lib):
    spec = CS.CASES["cavity_mrt"]
    g = gpu_solver(product, oracle_lib, spec, "fp32")
    with pytest.raises(product.LBMError):
        g.frame_fields(2)  # no step since the upload
    g.step(spec["tau"], spec["u"])
    with pytest.raises(product.LBMError):
        g.frame_fields(0)
    assert g.frame_fields(1)["rho"].shape == (spec["ny"], spec["nx"])
    g.close()


@pytest.mark.parametrize("kase,nx,ny", [(0, 201, 80), (1, 64, 64), (2, 48, 48)])
def test_dropin_writers_device_equals_host(product, tmp_path, kase, nx, ny):
    exe = tmp_path / "frame_drv"
    r = compile_dropin(os.path.join(HERE, "dropin", "frame_driver.cpp"), str(exe), flags=("-ffp-contract=off",))
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([str(exe), str(nx), str(ny), "40", "0.6", "0.1", str(kase), str(tmp_path / "out")],
                         capture_output=True, text=True, cwd=tmp_path, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "device_path=1 host_path=1" in run.stdout
    names = ["frames/frame_40.json", "frame_40.vtk"]
    for n in names:
        a = (tmp_path / "out" / "dev" / n).read_bytes()
        b = (tmp_path / "out" / "host" / n).read_bytes()
        assert len(a) > 100 and a == b, n
