"""C-ABI library: loads, exports every declared symbol, and its host-side
set-up arithmetic (masks, NACA profiles, point-in-polygon, wall distance,
bounce-back link list with q) is bit-exact against the oracle and the
reference's golden vectors.  No device call is made here."""
import os
import re

import numpy as np
import pytest

import cases as CS

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


def header_symbols():
    src = open(os.path.join(ROOT, "include", "lbm2d.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm2d_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(product):
    L = product.lib()
    syms = header_symbols()
    assert len(syms) >= 40
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(product.declared_symbols())


def test_create_without_gpu_fails_loudly(product):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is present")
    with pytest.raises(product.LBMError) as e:
        product.Solver(16, 16)
    assert e.value.code in (3, 6)


def test_equilibrium_and_geometry_kats(product):
    kat = np.load(os.path.join(GOLD, "kat.npz"))
    eq = [[product.equilibrium(i, rho, u, v) for i in range(9)]
          for rho, u, v in ((1.0, 0.0, 0.0), (1.2, 0.1, 0.05), (1.5, 0.12, -0.08), (0.9, -0.07, 0.11))]
    assert np.array_equal(np.array(eq), kat["equilibrium"])
    for series, n in ((12, 50), (2412, 60), (4415, 33)):
        assert np.array_equal(product.naca_coords(series, n), kat[f"naca_{series}_{n}"])
    p = product.transform_points(product.naca_coords(2412, 40), 30.0, 20.0, 36.0, 8.0)
    assert np.array_equal(p, kat["transform_2412"])
    pip = [product.point_in_polygon(x, y, p) for x, y in kat["pip_pts"]]
    assert np.array_equal(np.array(pip, np.uint8), kat["pip"])


@pytest.mark.parametrize("name", sorted(CS.IBM_CASES))
def test_ibm_points_and_airfoil_mask_bit_exact(product, name):
    """Lagrangian points (ImmersedBoundary::build_from_polygon) and the
    airfoil's point-in-polygon mask equal the reference's."""
    spec = CS.IBM_CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    nx, ny = spec["nx"], spec["ny"]
    poly = product.transform_points(product.naca_coords(spec["naca"], spec["npts"]), nx / 4, ny / 2, ny / 3.0,
                                    spec["aoa"])
    assert np.array_equal(poly, gold["poly"])
    assert np.array_equal(product.ibm_points_from_polygon(poly, spec["spacing"]), gold["points"])
    m = np.zeros(nx * ny, np.uint8)
    product.lib().lbm2d_mask_polygon(nx, ny, product._u8(m), product._d(np.ascontiguousarray(poly.reshape(-1))),
                                     len(poly))
    assert np.array_equal(m, gold["mask"])


@pytest.mark.parametrize("name", sorted(CS.CASES))
def test_masks_bit_exact_with_reference(product, name):
    """Masks made by the product's place_* helpers equal the reference's."""
    spec = CS.CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    nx, ny = spec["nx"], spec["ny"]
    m = np.zeros(nx * ny, np.uint8)
    L = product.lib()
    for op in spec["geometry"]:
        if op[0] == "walls":
            L.lbm2d_mask_walls(nx, ny, product._u8(m))
        elif op[0] == "cylinder":
            L.lbm2d_mask_cylinder(nx, ny, product._u8(m), *op[1:])
        elif op[0] in ("polygon", "naca"):
            xy = CS.polygon_of(op, product.naca_coords, product.transform_points).reshape(-1)
            L.lbm2d_mask_polygon(nx, ny, product._u8(m), product._d(xy), len(xy) // 2)
        elif op[0] == "row":
            m[op[1] * nx:(op[1] + 1) * nx] = 1
        elif op[0] == "mask":
            m[:] = np.maximum(m, CS.named_mask(op[1], nx, ny))
    assert np.array_equal(m, gold["mask"])


@pytest.mark.parametrize("name", ["ribs_les", "cavity_les"])
def test_wall_distance_matches_reference(product, name):
    spec = CS.CASES[name]
    gold = np.load(os.path.join(GOLD, f"{name}.npz"))
    wd = product.wall_distance(spec["nx"], spec["ny"], gold["mask"])
    assert np.array_equal(wd, gold["wall_dist"])


def _oracle_links(O, nx, ny, case_type, mask, setup):
    """Restated link enumeration of the reference's push streaming on the
    oracle: (node, i, q) for every fluid node whose neighbour is solid, with
    q from the oracle's compute_q (src/lbm_types.hpp:173-176)."""
    s = O.Solver(nx, ny)
    setup(s)
    cx = [0, 1, 0, -1, 0, 1, -1, -1, 1]
    cy = [0, 0, 1, 0, -1, 1, 1, -1, -1]
    out = {}
    for y in range(ny):
        for x in range(nx):
            n = y * nx + x
            if mask[n]:
                continue
            for i in range(1, 9):
                tx, ty = x + cx[i], (y + cy[i]) % ny
                if 0 <= tx < nx and mask[ty * nx + tx]:
                    out[(n, i)] = s.compute_q(x, y, i)
    s.close()
    return out


@pytest.mark.parametrize("kind", ["cylinder", "polygon"])
def test_boundary_link_q_bit_exact(product, oracle_lib, kind):
    nx, ny = 64, 40
    m = np.zeros(nx * ny, np.uint8)
    if kind == "cylinder":
        product.lib().lbm2d_mask_cylinder(nx, ny, product._u8(m), 20, 21, 7)
        links = product.boundary_links(nx, ny, 0, m, cylinder=(20, 21, 7), moving_wall=(0.01, 20.0, 21.0))
        ref = _oracle_links(oracle_lib, nx, ny, 0, m, lambda s: s.place_cylinder(20, 21, 7))
    else:
        poly = product.transform_points(product.naca_coords(2412, 40), 16.0, 20.0, 30.0, 10.0)
        xy = poly.reshape(-1)
        product.lib().lbm2d_mask_polygon(nx, ny, product._u8(m), product._d(xy), len(xy) // 2)
        links = product.boundary_links(nx, ny, 0, m, polygon=poly)
        ref = _oracle_links(oracle_lib, nx, ny, 0, m, lambda s: s.place_polygon(poly))
    got = {(int(n), int(i)): q for n, i, k, q in zip(links["node"], links["dir"], links["kind"], links["q"])
           if k == 2}
    assert set(got) == set(ref)
    assert len(got) > 20
    for key, q in ref.items():
        assert got[key] == q, key
    if kind == "cylinder":
        # Ladd wall velocity u = omega x r at the solid node (src/lbm_types.hpp:106-114)
        for n, i, k, uwx, uwy in zip(links["node"], links["dir"], links["kind"], links["uwx"], links["uwy"]):
            if k != 2:
                continue
            x, y = n % nx, n // nx
            px = x + [0, 1, 0, -1, 0, 1, -1, -1, 1][i]
            py = y + [0, 0, 1, 0, -1, 1, 1, -1, -1][i]
            assert uwx == -0.01 * (py - 21.0) and uwy == 0.01 * (px - 20.0)


def test_link_kinds_follow_case_wrap_rules(product):
    nx, ny = 12, 8
    m = np.zeros(nx * ny, np.uint8)
    m[0:nx] = 1  # bottom row solid
    # default case: x edges have no source (kind 3); periodic case: none
    d = product.boundary_links(nx, ny, 0, m)
    assert (d["kind"] == 3).sum() > 0 and set(np.unique(d["kind"])) <= {1, 3}
    r = product.boundary_links(nx, ny, 3, m)
    assert set(np.unique(r["kind"])) == {1}
    c = product.boundary_links(nx, ny, 1, m)
    assert set(np.unique(c["kind"])) == {1} and not c["force"].any()
