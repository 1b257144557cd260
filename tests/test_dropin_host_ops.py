"""The C++ drop-in's host-side node operators give the reference's bits.

Drivers can call mrt_collide and apply_bouzidi_bb (src/lbm.hpp:128-218,
:226-288) directly on host state.  The drop-in keeps both on the host in the
reference's operation order; this test compiles a small program against the
drop-in headers (tests/dropin/host_ops_driver.cpp, FP contraction off, no
device call), feeds it seeded inputs and compares every result with the
oracle -- the C restatement pinned bit-for-bit to the reference -- exactly:
  * mrt_collide with and without Smagorinsky, with and without Van Driest
    damping, over random nodes and relaxation times;
  * apply_bouzidi_bb on every fluid-to-solid link around a cylinder, for Mei
    and for classic Bouzidi + Ladd, with a static and a rotating wall.
CPU only."""
import os

import numpy as np
import pytest

from dropin_build import compile_dropin

HERE = os.path.dirname(os.path.abspath(__file__))
CX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])


@pytest.fixture(scope="module")
def driver(product, tmp_path_factory):
    exe = tmp_path_factory.mktemp("hostops") / "host_ops"
    r = compile_dropin(os.path.join(HERE, "dropin", "host_ops_driver.cpp"), str(exe), flags=("-ffp-contract=off",))
    assert r.returncode == 0, r.stderr[-3000:]
    return str(exe)


def _run(driver, tmp, nx, ny, mei, moving, geo, mask, f, links, mrt):
    inp, out = tmp / "in.bin", tmp / "out.bin"
    with open(inp, "wb") as fh:
        np.array([nx, ny, mei, moving, len(links), len(mrt)], "<i4").tofile(fh)
        np.array(geo, "<f8").tofile(fh)
        mask.astype(np.uint8).tofile(fh)
        f.astype("<f8").tofile(fh)
        np.array(links, "<i4").reshape(-1).tofile(fh)
        np.array(mrt, "<f8").reshape(-1).tofile(fh)
    import subprocess
    r = subprocess.run([driver, str(inp), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return np.fromfile(out, "<f8")


def _mrt_cases(rng, n=200):
    cases = []
    for k in range(n):
        rho = 1.0 + 0.05 * rng.standard_normal()
        u, v = 0.1 * rng.standard_normal(2)
        w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
        f = w * rho * (1 + 0.02 * rng.standard_normal(9))
        tau = rng.uniform(0.505, 1.9)
        cs_sq = [0.0, 0.01, 0.0144][k % 3]
        y_plus = [0.0, rng.uniform(0.1, 80.0)][k % 2]
        cases.append(np.concatenate([f, [rho, u, v, tau, cs_sq, y_plus]]))
    return cases


@pytest.mark.parametrize("mei,moving", [(1, 0), (0, 0), (1, 1), (0, 1)])
def test_host_operators_bit_exact(driver, oracle_lib, tmp_path, mei, moving):
    O = oracle_lib
    nx, ny = 48, 40
    ccx, ccy, rad = 20, 21, 7
    geo = [float(ccx), float(ccy), float(rad), 0.02 if moving else 0.0, float(ccx), float(ccy)]
    rng = np.random.default_rng(100 + 10 * mei + moving)
    s = O.Solver(nx, ny)
    s.set_case(O.CYLINDER)
    s.place_cylinder(ccx, ccy, rad)
    s.set_mei(bool(mei))
    if moving:
        s.set_moving_wall(True, geo[3], geo[4], geo[5])
    w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
    f = (np.tile(w, nx * ny) * (1.0 + 0.05 * rng.standard_normal(nx * ny * 9))).astype(np.float64)
    s.f[:] = f
    mask = s.obstacle.copy()
    links = []
    for y in range(1, ny - 1):
        for x in range(1, nx - 1):
            if mask[y * nx + x]:
                continue
            for i in range(1, 9):
                if mask[(y + CY[i]) * nx + (x + CX[i])]:
                    links.append((x, y, i))
    assert len(links) > 40
    mrt = _mrt_cases(rng)
    got = _run(driver, tmp_path, nx, ny, mei, moving, geo, mask, f, links, mrt)
    want_links = np.array([O.lib()[0].or_interp_bb_link(s.h, x, y, i) for x, y, i in links])
    s.close()
    assert np.array_equal(got[:len(links)], want_links)
    L = O.lib()[0]
    want_mrt = []
    for c in mrt:
        fn = np.ascontiguousarray(c[:9])
        rho, u, v, tau, cs_sq, y_plus = c[9:]
        ss, sb, sn = 1.0 / tau, 1.2, 1.0
        ss = 0.5 if ss < 0.5 else (1.99 if ss > 1.99 else ss)
        L.or_mrt_collide(fn.ctypes.data_as(O._DP), rho, u, v, ss, sb, sn, cs_sq, tau, y_plus)
        want_mrt.append(fn)
    assert np.array_equal(got[len(links):].reshape(-1, 9), np.array(want_mrt))
