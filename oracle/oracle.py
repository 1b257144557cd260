"""ctypes front end of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle.so`` (the C restatement in ``lbm_oracle.c``)
or, in this development container only, ``oracle/_ref/libref.so`` (the
reference solver's own headers driven by ``ref_harness.cpp``).  Both expose
the same call surface; :class:`Solver` hides the difference so one case
specification can be run on either.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this
module.  The product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "_build", "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libref.so")

# Case numbering of the reference (src/lbm_types.hpp:20-23).
CYLINDER, CAVITY, STEP, RIBS, URBAN_CANYON, DOWNWASH, SQUARE_CYLINDER, FLAT_PLATE, \
    SPORTS_BALL, PERIODIC_HILLS, CYLINDER_NEAR_WALL, SIDE_BY_SIDE, ROTATING_CYLINDER, \
    ORIFICE_PLATE = range(14)
MRT, BGK = 0, 1

_D = C.c_double
_I = C.c_int
_P = C.c_void_p
_DP = C.POINTER(C.c_double)


def build(ref_src: str | None = None, with_ref: bool = False) -> None:
    """Compile the oracle (and the reference harness when its sources exist)."""
    cmd = ["make", "-s", "-C", HERE]
    subprocess.run(cmd, check=True)
    if with_ref and ref_src and os.path.isdir(ref_src):
        subprocess.run(cmd + ["ref", f"REF_SRC={ref_src}"], check=True)


def _load(path: str, prefix: str) -> C.CDLL:
    lib = C.CDLL(path)
    stateful = prefix == "or_"
    sig = {
        "create": ([_I, _I], _P if stateful else _I),
        "destroy": ([], None),
        "set_case": ([_I, _I, _I, _D], None),
        "set_thermal": ([_I, _D, _D, _D, _D, _D], None),
        "set_body_force": ([_D], None),
        "set_moving_wall": ([_I, _D, _D, _D], None),
        "set_mei": ([_I], None),
        "f": ([], _DP), "g": ([], _DP), "fx": ([], _DP), "fy": ([], _DP),
        "wall_dist": ([], _DP), "obstacle": ([], C.POINTER(C.c_uint8)),
        "place_walls": ([], None),
        "place_cylinder": ([_I, _I, _I], None),
        "place_polygon": ([_DP, _I], None),
        "compute_wall_distance": ([], None),
        "compute_q": ([_D, _D, _I], _D),
        "step": ([_D, _D], None),
        "force_sums": ([_DP, _DP], None),
        "thermal_hook": ([_I, _D, _D], None),
        "init_cylinder_wake": ([_D, _I, C.c_uint, _D], None),
        "init_uniform": ([_D, _D, _D], None),
        "init_thermal_uniform": ([_D, _D, _D], None),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, prefix + name)
        if stateful and name != "create":
            args = [_P] + args
        fn.argtypes = args
        fn.restype = res
    free = {
        "naca_coords": ([_I, _I, _DP], _I),
        "transform_points": ([_DP, _I, _D, _D, _D, _D], None),
        "point_in_polygon": ([_D, _D, _DP, _I], _I),
        "equilibrium": ([_I, _D, _D, _D], _D),
    }
    for name, (args, res) in free.items():
        fn = getattr(lib, prefix + name)
        fn.argtypes = args
        fn.restype = res
    # immersed boundary: the harness wraps the reference's ImmersedBoundary,
    # the restatement takes the points explicitly
    if stateful:
        ibm = {
            "or_ibm_points_from_polygon": ([_DP, _I, _D, _DP, _DP, _I], _I),
            "or_ibm_set": ([_P, _DP, _DP, _I, _D, _D, _D], None),
            "or_ibm_step": ([_P, _D, _D], None),
            "or_ibm_lagrangian": ([_P, _DP, _DP, _DP, _DP], None),
            "or_ibm_kernel": ([_D, _D], _D),
            "or_interp_bb_link": ([_P, _I, _I, _I], _D),
            "or_mrt_collide": ([_DP, _D, _D, _D, _D, _D, _D, _D, _D, _D], None),
        }
    else:
        ibm = {
            "ref_ibm_from_polygon": ([_DP, _I, _D], _I),
            "ref_ibm_points": ([_DP, _DP], None),
            "ref_ibm_set_dt": ([_D], None),
            "ref_ibm_step": ([_D, _D], None),
            "ref_ibm_lagrangian": ([_DP, _DP, _DP, _DP], None),
            "ref_ibm_kernel": ([_D, _D], _D),
        }
    for name, (args, res) in ibm.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


_LIBS: dict[str, C.CDLL] = {}


def lib(kind: str = "oracle") -> tuple[C.CDLL, str]:
    path, prefix = (LIB_ORACLE, "or_") if kind == "oracle" else (LIB_REF, "ref_")
    if kind not in _LIBS:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built")
        _LIBS[kind] = _load(path, prefix)
    return _LIBS[kind], prefix


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_DP)


class Solver:
    """One FP64 solver instance of the oracle (or of the reference harness)."""

    def __init__(self, nx: int, ny: int, kind: str = "oracle"):
        self.lib, self.prefix = lib(kind)
        self.kind = kind
        self.nx, self.ny = nx, ny
        if kind == "oracle":
            self.h = self.lib.or_create(nx, ny)
        else:
            self.lib.ref_create(nx, ny)
            self.h = None

    def _c(self, name, *args):
        fn = getattr(self.lib, self.prefix + name)
        return fn(self.h, *args) if self.h is not None else fn(*args)

    def close(self):
        if self.h is not None:
            self.lib.or_destroy(self.h)
            self.h = None
        elif self.kind == "ref":
            self.lib.ref_destroy()
            self.kind = "closed"

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # arrays (views into the C state; copy before the next step if kept)
    def _view(self, name, count, dtype=np.float64):
        p = self._c(name)
        return np.ctypeslib.as_array(p, shape=(count,)).view(dtype)

    @property
    def f(self):
        return self._view("f", self.nx * self.ny * 9)

    @property
    def g(self):
        return self._view("g", self.nx * self.ny * 9)

    @property
    def fx(self):
        return self._view("fx", self.nx * self.ny)

    @property
    def fy(self):
        return self._view("fy", self.nx * self.ny)

    @property
    def wall_dist(self):
        return self._view("wall_dist", self.nx * self.ny)

    @property
    def obstacle(self):
        p = self._c("obstacle")
        return np.ctypeslib.as_array(p, shape=(self.nx * self.ny,))

    def set_case(self, case_type, collision=MRT, use_les=False, cs=0.12):
        self._c("set_case", int(case_type), int(collision), int(bool(use_les)), float(cs))

    def set_thermal(self, use, T_ref=1.0, alpha=0.1666666667, omega_k=1.0, beta=0.0, g_buoyancy=0.0):
        self._c("set_thermal", int(bool(use)), T_ref, alpha, omega_k, beta, g_buoyancy)

    def set_body_force(self, fx):
        self._c("set_body_force", float(fx))

    def set_moving_wall(self, on, omega=0.0, rcx=0.0, rcy=0.0):
        self._c("set_moving_wall", int(bool(on)), omega, rcx, rcy)

    def set_mei(self, on):
        self._c("set_mei", int(bool(on)))

    def place_walls(self):
        self._c("place_walls")

    def place_cylinder(self, cx, cy, r):
        self._c("place_cylinder", int(cx), int(cy), int(r))

    def place_polygon(self, xy):
        xy = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        self._c("place_polygon", _dptr(xy), len(xy) // 2)

    def compute_wall_distance(self):
        self._c("compute_wall_distance")

    def compute_q(self, xf, yf, i):
        return self._c("compute_q", float(xf), float(yf), int(i))

    def step(self, tau, u_in, n=1, hook=None):
        for _ in range(n):
            self._c("step", float(tau), float(u_in))
            if hook is not None:
                self.thermal_hook(*hook)

    def force_sums(self):
        a, b = _D(), _D()
        self._c("force_sums", C.byref(a), C.byref(b))
        return a.value, b.value

    def thermal_hook(self, kind, Ta, Tb=0.0):
        self._c("thermal_hook", int(kind), float(Ta), float(Tb))

    def init_cylinder_wake(self, u_in, cx_cyl, seed=42, amp=1e-4):
        self._c("init_cylinder_wake", float(u_in), int(cx_cyl), int(seed), float(amp))

    def init_uniform(self, rho, u, v):
        self._c("init_uniform", float(rho), float(u), float(v))

    def init_thermal_uniform(self, T, u, v):
        self._c("init_thermal_uniform", float(T), float(u), float(v))

    # immersed boundary (src/ibm.hpp, driven as src/airfoil_ibm.cpp:121-176)
    def ibm_from_polygon(self, xy, spacing=1.0, dt=1.0):
        """Lagrangian points of ImmersedBoundary::build_from_polygon, installed
        for ibm_step; returns them as an (n, 2) array."""
        a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
        if self.kind == "ref":
            n = self.lib.ref_ibm_from_polygon(_dptr(a), len(a) // 2, float(spacing))
            X, Y = np.zeros(n), np.zeros(n)
            self.lib.ref_ibm_points(_dptr(X), _dptr(Y))
            self.lib.ref_ibm_set_dt(float(dt))
        else:
            X, Y = ibm_points_from_polygon(a.reshape(-1, 2), spacing).T.copy()
            self.lib.or_ibm_set(self.h, _dptr(X), _dptr(Y), len(X), float(dt), 0.0, 0.0)
        self._ibm_n = len(X)
        return np.stack([X, Y], 1)

    def ibm_step(self, tau, u_in, n=1):
        for _ in range(n):
            self._c("ibm_step", float(tau), float(u_in))

    def ibm_lagrangian(self):
        """(U, V, FX, FY) at the Lagrangian points after the last ibm_step."""
        out = [np.zeros(self._ibm_n) for _ in range(4)]
        self._c("ibm_lagrangian", *(_dptr(a) for a in out))
        return tuple(out)


def ibm_points_from_polygon(xy, spacing=1.0) -> np.ndarray:
    """ImmersedBoundary::build_from_polygon (src/ibm.hpp:42-69), restated."""
    L, _ = lib("oracle")
    a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
    n = L.or_ibm_points_from_polygon(_dptr(a), len(a) // 2, float(spacing), None, None, 0)
    X, Y = np.zeros(n), np.zeros(n)
    L.or_ibm_points_from_polygon(_dptr(a), len(a) // 2, float(spacing), _dptr(X), _dptr(Y), n)
    return np.stack([X, Y], 1)


def ibm_kernel(dx, dy, kind: str = "oracle") -> float:
    L, p = lib(kind)
    return getattr(L, p + "ibm_kernel")(float(dx), float(dy))


def naca_coords(series: int, n: int = 200, kind: str = "oracle") -> np.ndarray:
    L, p = lib(kind)
    out = np.zeros(2 * (2 * n), dtype=np.float64)
    k = getattr(L, p + "naca_coords")(series, n, _dptr(out))
    return out[: 2 * k].reshape(-1, 2).copy()


def transform_points(xy: np.ndarray, cx, cy, scale, angle_deg, kind: str = "oracle") -> np.ndarray:
    L, p = lib(kind)
    a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1).copy()
    getattr(L, p + "transform_points")(_dptr(a), len(a) // 2, float(cx), float(cy), float(scale), float(angle_deg))
    return a.reshape(-1, 2)


def point_in_polygon(px, py, xy, kind: str = "oracle") -> bool:
    L, p = lib(kind)
    a = np.ascontiguousarray(xy, dtype=np.float64).reshape(-1)
    return bool(getattr(L, p + "point_in_polygon")(float(px), float(py), _dptr(a), len(a) // 2))


def equilibrium(i, rho, u, v, kind: str = "oracle") -> float:
    L, p = lib(kind)
    return getattr(L, p + "equilibrium")(int(i), float(rho), float(u), float(v))
