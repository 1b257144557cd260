"""The bench's seeded synthetic workloads against the shapes, sizes and value
distributions they stand in for (CPU only):

* the large-domain channel: periodic-x channel with solid rows y = 0 and
  y = NY-1 and 64 non-overlapping circles of radius 8-40 (4096x4096 and
  8192x4096), pinned by a digest so that bench figures stay comparable;
* 256 uneven batch instances: sides log-uniform in [64, 1024], aspect 1-3,
  cavity / step / cylinder, Re in [50, 1000], about 30% heated cavities with
  Ra up to 1e5;
* the serving stream: grids 128x64 to 2048x768 (cavities square with the
  same node count), cavity / backward step / cylinder / two side-by-side
  cylinders with S/D in [2, 5], Re in [50, 2000], step budgets 1k-50k.
"""
import hashlib
import math

import numpy as np
import pytest

import bench as B


@pytest.mark.parametrize("nx,ny,digest", [(4096, 4096, "0a914b984597f7eb"), (8192, 4096, None)])
def test_channel_geometry(nx, ny, digest):
    mask, circles = B.make_geometry(nx, ny)
    m = mask.reshape(ny, nx)
    assert len(circles) == B.N_CIRCLES == 64
    assert m[0].all() and m[ny - 1].all()
    for k, (cx, cy, r) in enumerate(circles):
        assert B.RMIN <= r <= B.RMAX
        assert r + 2 <= cx <= nx - r - 3 and r + 3 <= cy <= ny - r - 3
        for cx2, cy2, r2 in circles[k + 1:]:
            assert math.hypot(cx - cx2, cy - cy2) > r + r2  # non-overlapping
        # the reference's place_cylinder rule, sqrt(dx^2 + dy^2) < r, on the circle's box
        yy, xx = np.mgrid[cy - r - 1:cy + r + 2, cx - r - 1:cx + r + 2]
        inside = np.sqrt((xx - cx).astype(np.float64) ** 2 + (yy - cy).astype(np.float64) ** 2) < r
        assert np.array_equal(m[cy - r - 1:cy + r + 2, cx - r - 1:cx + r + 2] != 0, inside)
    mask2, circles2 = B.make_geometry(nx, ny)  # seeded: the same workload every run
    assert np.array_equal(mask, mask2) and circles == circles2
    if digest:
        assert hashlib.sha256(mask.tobytes()).hexdigest()[:16] == digest


def test_batch_instances():
    inst = B._c4_instances()
    assert len(inst) == 256
    thermal = [i for i in inst if i["geometry"] == 4]
    assert 0.22 <= len(thermal) / len(inst) <= 0.38
    for i in thermal:
        assert 64 <= i["nx"] == i["ny"] <= 1024 and 1e3 <= i["param"] <= 1e5
    rest = [i for i in inst if i["geometry"] != 4]
    assert {i["geometry"] for i in rest} == {0, 1, 2}
    for i in rest:
        assert 64 <= i["ny"] <= 1024 and i["ny"] <= i["nx"] <= 3 * i["ny"] + 1
        assert 50.0 <= i["re"] <= 1000.0
        if i["geometry"] == 0:
            assert i["nx"] == i["ny"]
    sides = np.log([i["ny"] for i in inst])  # log-uniform sides: spread over the whole range
    assert sides.min() < math.log(80) and sides.max() > math.log(800)


def test_serving_requests():
    req = B._c5_requests(200)
    assert len(req) == 200
    assert {r["geometry"] for r in req} == {0, 1, 2, 3}
    for r in req:
        # cavities are square (the reference's cavity driver forces NX = NY)
        # with the node count of the grid drawn for them
        assert 128 * 64 * 0.99 <= r["nx"] * r["ny"] <= 2048 * 768
        if r["geometry"] == 0:
            assert r["nx"] == r["ny"]
        else:
            assert 128 <= r["nx"] <= 2048 and 64 <= r["ny"] <= 768
        assert 50.0 <= r["re"] <= 2000.0
        assert 1000 <= r["steps"] <= 50000
        if r["geometry"] == 3:
            assert 2.0 <= r["param"] <= 5.0
    assert B._c5_requests(200) == req


def test_cpu_leg_picks_reference_build_or_port(oracle_lib, monkeypatch, tmp_path):
    """The CPU legs time the reference's own compiled step when that build
    loads on the host, and fall back to the restatement when it is missing
    or cannot load (an x86 build on an Arm host)."""
    import os

    O = oracle_lib
    if os.path.exists(O.LIB_REF):
        assert B._cpu_impl()[:2] == ("ref", "reference")
    monkeypatch.setattr(O, "LIB_REF", str(tmp_path / "missing.so"))
    assert B._cpu_impl()[:2] == ("oracle", "port")
    bad = tmp_path / "bad.so"
    bad.write_bytes(b"not a shared object")
    monkeypatch.setattr(O, "LIB_REF", str(bad))
    monkeypatch.setattr(O, "_LIBS", {k: v for k, v in O._LIBS.items() if k == "oracle"})  # no cached load
    assert B._cpu_impl()[:2] == ("oracle", "port")
