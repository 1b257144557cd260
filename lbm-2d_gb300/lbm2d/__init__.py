"""Python binding of liblbm2d (the GB300 D2Q9 lattice-Boltzmann step).

A thin ctypes layer over the C-ABI in include/lbm2d.h.  :class:`Solver`
mirrors the reference's solver surface (LBMCapabilities + execute_time_step +
place_* helpers of src/lbm.hpp / src/lbm_types.hpp) with host arrays in the
reference's layouts, so tests and benchmarks read like the reference's own.

There is no CPU fallback: every compute call goes to the CUDA library, and
constructing a Solver without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._build import LIB, build as _build_lib, needs_build  # noqa: F401

CYLINDER, CAVITY, STEP, RIBS, URBAN_CANYON, DOWNWASH, SQUARE_CYLINDER, FLAT_PLATE, \
    SPORTS_BALL, PERIODIC_HILLS, CYLINDER_NEAR_WALL, SIDE_BY_SIDE, ROTATING_CYLINDER, \
    ORIFICE_PLATE = range(14)
MRT, BGK = 0, 1
STORAGE = {"fp32": 0, "fp16": 1, "bf16": 2, "fp64": 3}
BYTES_PER_POP = {"fp32": 4, "fp16": 2, "bf16": 2, "fp64": 8}
HOOK_NONE, HOOK_HEATED_CAVITY, HOOK_HEATED_SOLIDS = 0, 1, 2
KERNEL_SCALAR, KERNEL_PAIR, KERNEL_ROWS, KERNEL_TILES = 0, 1, 2, 3

ERRORS = {1: "invalid argument", 2: "out of device memory", 3: "CUDA error", 4: "non-finite density",
          5: "call out of order", 6: "no CUDA device", 7: "device wait timed out"}


class LBMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"lbm2d error {code} ({ERRORS.get(code, '?')}): {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("case_type", C.c_int), ("collision", C.c_int),
                ("use_les", C.c_int), ("cs", C.c_double), ("storage", C.c_int), ("device", C.c_int)]


class Info(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("storage", C.c_int), ("bytes_per_update", C.c_double),
                ("device_bytes", C.c_size_t), ("n_boundary_nodes", C.c_int), ("n_force_nodes", C.c_int),
                ("steps_done", C.c_longlong), ("block_x", C.c_int), ("block_y", C.c_int), ("kernel", C.c_int)]


class BBGeometry(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("radius", C.c_double),
                ("poly", C.POINTER(C.c_double)), ("n_poly", C.c_int), ("has_moving_wall", C.c_int),
                ("omega", C.c_double), ("rot_cx", C.c_double), ("rot_cy", C.c_double)]


class Request(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("geometry", C.c_int), ("re", C.c_double),
                ("param", C.c_double), ("u", C.c_double), ("steps", C.c_int), ("storage", C.c_int)]


class Result(C.Structure):
    _fields_ = [("id", C.c_longlong), ("status", C.c_int), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double), ("steps", C.c_longlong), ("nodes", C.c_longlong), ("fx", C.c_double),
                ("fy", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("finished", C.c_longlong), ("queued", C.c_longlong),
                ("active", C.c_longlong), ("busy_s", C.c_double), ("lattice_updates", C.c_longlong),
                ("device_bytes_in_use", C.c_double), ("ticks", C.c_longlong), ("member_ticks", C.c_longlong),
                ("setup_s", C.c_double), ("gpu_s", C.c_double), ("call_s", C.c_double), ("wait_s", C.c_double),
                ("retire_s", C.c_double), ("join_s", C.c_double)]


class ForceStats(C.Structure):
    _fields_ = [("mean_v1", C.c_double), ("mean_v2", C.c_double), ("std_v2", C.c_double), ("st", C.c_double),
                ("n_skip", C.c_int)]


GEOM_CAVITY, GEOM_STEP, GEOM_CYLINDER, GEOM_SIDE_BY_SIDE, GEOM_HEATED_CAVITY = range(5)

_D, _I, _P = C.c_double, C.c_int, C.c_void_p
_DP = C.POINTER(C.c_double)
_U8P = C.POINTER(C.c_uint8)

_SIGS = {
    "lbm2d_create": ([C.POINTER(Config), C.POINTER(_P)], _I),
    "lbm2d_destroy": ([_P], _I),
    "lbm2d_last_error": ([_P], C.c_char_p),
    "lbm2d_global_error": ([], C.c_char_p),
    "lbm2d_set_case": ([_P, _I, _I, _I, _D], _I),
    "lbm2d_set_mask": ([_P, _U8P], _I),
    "lbm2d_set_bb_cylinder": ([_P, _D, _D, _D], _I),
    "lbm2d_set_bb_polygon": ([_P, _DP, _I], _I),
    "lbm2d_set_moving_wall": ([_P, _I, _D, _D, _D], _I),
    "lbm2d_set_mei": ([_P, _I], _I),
    "lbm2d_set_body_force": ([_P, _D], _I),
    "lbm2d_set_thermal": ([_P, _I, _D, _D, _D, _D, _D], _I),
    "lbm2d_set_thermal_hook": ([_P, _I, _D, _D], _I),
    "lbm2d_upload_f": ([_P, _DP], _I),
    "lbm2d_upload_g": ([_P, _DP], _I),
    "lbm2d_upload_f_device": ([_P, _P], _I),
    "lbm2d_download_f_device": ([_P, _P], _I),
    "lbm2d_step": ([_P, _D, _D, _I], _I),
    "lbm2d_init_equilibrium": ([_P, _D, _D, _D, _D], _I),
    "lbm2d_step_noalloc": ([_P, _D, _D, _I], _I),
    "lbm2d_force_sums": ([_P, _DP, _DP], _I),
    "lbm2d_force_history": ([_P, _DP, _DP, _I, C.POINTER(_I)], _I),
    "lbm2d_force_history_reset": ([_P], _I),
    "lbm2d_download_f": ([_P, _DP], _I),
    "lbm2d_download_g": ([_P, _DP], _I),
    "lbm2d_download_force_field": ([_P, _DP, _DP], _I),
    "lbm2d_download_macros": ([_P, _DP, _DP, _DP, _DP], _I),
    "lbm2d_download_wall_dist": ([_P, _DP], _I),
    "lbm2d_frame_fields": ([_P, _I, _I, _D, _DP, _DP, _DP, _DP, _DP, _DP, _U8P], _I),
    "lbm2d_diagnostics": ([_P, _DP, _DP, _DP, _DP], _I),
    "lbm2d_synchronize": ([_P], _I),
    "lbm2d_get_info": ([_P, C.POINTER(Info)], _I),
    "lbm2d_set_block": ([_P, _I, _I], _I),
    "lbm2d_set_kernel_variant": ([_P, _I], _I),
    "lbm2d_set_wait_limit": ([_P, C.c_longlong], _I),
    "lbm2d_stream": ([_P], _P),
    "lbm2d_set_profiling": ([_P, _I], _I),
    "lbm2d_profile": ([_P, _DP, C.POINTER(C.c_longlong)], _I),
    "lbm2d_launch_count": ([_P], C.c_longlong),
    "lbm2d_batch_create": ([_I, C.POINTER(_P)], _I),
    "lbm2d_batch_destroy": ([_P], _I),
    "lbm2d_batch_last_error": ([_P], C.c_char_p),
    "lbm2d_batch_add": ([_P, _P, _D, _D], _I),
    "lbm2d_batch_remove": ([_P, _P], _I),
    "lbm2d_batch_set_params": ([_P, _P, _D, _D], _I),
    "lbm2d_batch_size": ([_P], _I),
    "lbm2d_batch_set_budget": ([_P, _P, C.c_longlong], _I),
    "lbm2d_batch_budget": ([_P, _P], C.c_longlong),
    "lbm2d_batch_step": ([_P, _I], _I),
    "lbm2d_batch_synchronize": ([_P], _I),
    "lbm2d_batch_set_block": ([_P, _I, _I], _I),
    "lbm2d_batch_stream": ([_P], _P),
    "lbm2d_batch_launch_count": ([_P], C.c_longlong),
    "lbm2d_autotune": ([_P, _I, _D, _D, C.POINTER(_I), C.POINTER(_I)], _I),
    "lbm2d_server_create": ([_I, _D, _I, _I, C.POINTER(_P)], _I),
    "lbm2d_server_create_ex": ([_I, _D, _I, _I, _I, C.POINTER(_P)], _I),
    "lbm2d_server_submit": ([_P, C.POINTER(Request), C.POINTER(C.c_longlong)], _I),
    "lbm2d_server_submit_state": ([_P, C.POINTER(Request), _DP, _DP, _DP, C.POINTER(C.c_longlong)], _I),
    "lbm2d_server_wait": ([_P, C.c_longlong, _D], _I),
    "lbm2d_server_results": ([_P, C.POINTER(Result), _I, C.POINTER(_I)], _I),
    "lbm2d_server_stats": ([_P, C.POINTER(ServerStats)], _I),
    "lbm2d_server_destroy": ([_P], _I),
    "lbm2d_batch_autotune": ([_P, _I, C.POINTER(_I), C.POINTER(_I)], _I),
    # host services
    "lbm2d_equilibrium": ([_I, _D, _D, _D], _D),
    "lbm2d_mask_walls": ([_I, _I, _U8P], _I),
    "lbm2d_mask_cylinder": ([_I, _I, _U8P, _I, _I, _I], _I),
    "lbm2d_mask_polygon": ([_I, _I, _U8P, _DP, _I], _I),
    "lbm2d_point_in_polygon": ([_D, _D, _DP, _I], _I),
    "lbm2d_naca_coords": ([_I, _I, _DP], _I),
    "lbm2d_transform_points": ([_DP, _I, _D, _D, _D, _D], _I),
    "lbm2d_wall_distance": ([_I, _I, _U8P, _DP], _I),
    "lbm2d_ibm_points_from_polygon": ([_DP, _I, _D, _DP, _DP, _I], _I),
    "lbm2d_set_ibm": ([_P, _DP, _DP, _I, _D, _D, _D], _I),
    "lbm2d_ibm_lagrangian": ([_P, _DP, _DP, _DP, _DP], _I),
    "lbm2d_force_stats": ([_DP, _DP, _I, _D, C.POINTER(ForceStats)], _I),
    "lbm2d_boundary_links": ([_I, _I, _I, _U8P, C.POINTER(BBGeometry), _I, C.POINTER(C.c_int32),
                              C.POINTER(C.c_int8), C.POINTER(C.c_int8), _DP, _DP, _DP,
                              C.POINTER(C.c_int8), C.POINTER(_I)], _I),
}

_lib: C.CDLL | None = None


def build(force: bool = False, quiet: bool = False) -> str:
    return _build_lib(force=force, quiet=quiet)


def lib() -> C.CDLL:
    """Load liblbm2d.so (in-tree).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is not built; call lbm2d.build() first")
        L = C.CDLL(LIB)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def declared_symbols() -> list[str]:
    return list(_SIGS)


def _d(a: np.ndarray):
    return a.ctypes.data_as(_DP)


def _u8(a: np.ndarray):
    return a.ctypes.data_as(_U8P)


# ---------------------------------------------------------------- host services
def equilibrium(i, rho, u, v) -> float:
    return lib().lbm2d_equilibrium(int(i), float(rho), float(u), float(v))


def equilibrium_field(nx, ny, rho, u, v) -> np.ndarray:
    """Uniform equilibrium populations [nx*ny*9] (FP64 AoS), as the drivers' init loops."""
    one = np.array([equilibrium(i, rho, u, v) for i in range(9)])
    return np.tile(one, nx * ny)


def naca_coords(series: int, n: int = 200) -> np.ndarray:
    out = np.zeros(2 * (2 * n), np.float64)
    k = lib().lbm2d_naca_coords(int(series), int(n), _d(out))
    return out[: 2 * k].reshape(-1, 2).copy()


def transform_points(xy, cx, cy, scale, angle_deg) -> np.ndarray:
    a = np.ascontiguousarray(xy, np.float64).reshape(-1).copy()
    lib().lbm2d_transform_points(_d(a), len(a) // 2, float(cx), float(cy), float(scale), float(angle_deg))
    return a.reshape(-1, 2)


def point_in_polygon(px, py, xy) -> bool:
    a = np.ascontiguousarray(xy, np.float64).reshape(-1)
    return bool(lib().lbm2d_point_in_polygon(float(px), float(py), _d(a), len(a) // 2))


def force_stats(v1, v2, dt=1.0) -> dict:
    """Mean Cd/Cl (or Fx/Fy), std of the lift and the shedding frequency, as
    the reference's post-processing computes them."""
    a = np.ascontiguousarray(v1, np.float64)
    b = np.ascontiguousarray(v2, np.float64)
    st = ForceStats()
    rc = lib().lbm2d_force_stats(_d(a), _d(b), len(a), float(dt), C.byref(st))
    if rc:
        raise LBMError(rc, "force_stats")
    return {k: getattr(st, k) for k, _ in ForceStats._fields_}


def drag_lift_coefficients(fx, fy, length_scale, u):
    """Cd, Cl = 2 F / (D u^2) as the cylinder driver normalises (src/main.cpp:112-115)."""
    k = 2.0 / (length_scale * u * u)
    return np.asarray(fx) * k, np.asarray(fy) * k


def wall_distance(nx, ny, mask) -> np.ndarray:
    m = np.ascontiguousarray(mask, np.uint8).reshape(-1)
    out = np.zeros(nx * ny, np.float64)
    lib().lbm2d_wall_distance(nx, ny, _u8(m), _d(out))
    return out


def ibm_points_from_polygon(xy, spacing=1.0) -> np.ndarray:
    """Lagrangian points of ImmersedBoundary::build_from_polygon as an (n, 2)
    array."""
    a = np.ascontiguousarray(xy, np.float64).reshape(-1)
    L = lib()
    n = L.lbm2d_ibm_points_from_polygon(_d(a), len(a) // 2, float(spacing), None, None, 0)
    X, Y = np.zeros(n), np.zeros(n)
    L.lbm2d_ibm_points_from_polygon(_d(a), len(a) // 2, float(spacing), _d(X), _d(Y), n)
    return np.stack([X, Y], 1)


def boundary_links(nx, ny, case_type, mask, cylinder=None, polygon=None, moving_wall=None) -> dict:
    """The reference's bounce-back link list for a mask (see include/lbm2d.h)."""
    m = np.ascontiguousarray(mask, np.uint8).reshape(-1)
    g = BBGeometry()
    keep = None
    if cylinder is not None:
        g.cx, g.cy, g.radius = map(float, cylinder)
    if polygon is not None:
        keep = np.ascontiguousarray(polygon, np.float64).reshape(-1)
        g.poly = _d(keep)
        g.n_poly = len(keep) // 2
    if moving_wall is not None:
        g.has_moving_wall = 1
        g.omega, g.rot_cx, g.rot_cy = map(float, moving_wall)
    cnt = C.c_int(0)
    L = lib()
    rc = L.lbm2d_boundary_links(nx, ny, case_type, _u8(m), C.byref(g), 0, None, None, None, None, None, None,
                                None, C.byref(cnt))
    if rc:
        raise LBMError(rc, "boundary_links")
    n = cnt.value
    out = dict(node=np.zeros(n, np.int32), dir=np.zeros(n, np.int8), kind=np.zeros(n, np.int8),
               q=np.zeros(n), uwx=np.zeros(n), uwy=np.zeros(n), force=np.zeros(n, np.int8))
    L.lbm2d_boundary_links(nx, ny, case_type, _u8(m), C.byref(g), n,
                           out["node"].ctypes.data_as(C.POINTER(C.c_int32)),
                           out["dir"].ctypes.data_as(C.POINTER(C.c_int8)),
                           out["kind"].ctypes.data_as(C.POINTER(C.c_int8)),
                           _d(out["q"]), _d(out["uwx"]), _d(out["uwy"]),
                           out["force"].ctypes.data_as(C.POINTER(C.c_int8)), C.byref(cnt))
    del keep
    return out


# ---------------------------------------------------------------- solver
class Solver:
    """One GPU solver instance (the reference's LBMCapabilities + globals)."""

    def __init__(self, nx: int, ny: int, case_type: int = CYLINDER, collision: int = MRT, use_les: bool = False,
                 cs: float = 0.12, storage: str = "fp32", device: int = 0):
        L = lib()
        cfg = Config(nx, ny, case_type, collision, int(bool(use_les)), cs, STORAGE[storage], device)
        h = _P()
        rc = L.lbm2d_create(C.byref(cfg), C.byref(h))
        if rc:
            raise LBMError(rc, L.lbm2d_global_error().decode())
        self.h = h
        self.L = L
        self.nx, self.ny = nx, ny
        self.storage = storage
        self._mask = np.zeros(nx * ny, np.uint8)
        self._ibm_n = 0

    # -- plumbing
    def _ck(self, rc):
        if rc:
            raise LBMError(rc, self.L.lbm2d_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm2d_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def obstacle(self) -> np.ndarray:
        """Solid mask (read-only view); change it with set_mask or place_*."""
        v = self._mask.view()
        v.flags.writeable = False
        return v

    def set_mask(self, mask):
        """LBMCapabilities::obstacle: one byte per node, pushed to the solver."""
        m = np.ascontiguousarray(mask, np.uint8).reshape(-1)
        assert m.size == self.nx * self.ny
        self._mask = (m != 0).astype(np.uint8)
        self._ck(self.L.lbm2d_set_mask(self.h, _u8(self._mask)))

    # -- configuration (reference names)
    def set_case(self, case_type, collision=MRT, use_les=False, cs=0.12):
        self._ck(self.L.lbm2d_set_case(self.h, int(case_type), int(collision), int(bool(use_les)), float(cs)))

    def place_walls(self):
        m = self._mask.copy()
        self._ck(self.L.lbm2d_mask_walls(self.nx, self.ny, _u8(m)))
        self.set_mask(m)

    def place_cylinder(self, cx, cy, r):
        m = self._mask.copy()
        self._ck(self.L.lbm2d_mask_cylinder(self.nx, self.ny, _u8(m), int(cx), int(cy), int(r)))
        self.set_mask(m)
        self.set_bb_cylinder(cx, cy, r)

    def place_polygon(self, xy):
        a = np.ascontiguousarray(xy, np.float64).reshape(-1)
        m = self._mask.copy()
        self._ck(self.L.lbm2d_mask_polygon(self.nx, self.ny, _u8(m), _d(a), len(a) // 2))
        self.set_mask(m)
        self.set_bb_polygon(a)

    def set_bb_cylinder(self, cx, cy, r):
        self._ck(self.L.lbm2d_set_bb_cylinder(self.h, float(cx), float(cy), float(r)))

    def set_bb_polygon(self, xy):
        a = np.ascontiguousarray(xy, np.float64).reshape(-1)
        self._ck(self.L.lbm2d_set_bb_polygon(self.h, _d(a), len(a) // 2))

    def set_moving_wall(self, on, omega=0.0, rcx=0.0, rcy=0.0):
        self._ck(self.L.lbm2d_set_moving_wall(self.h, int(bool(on)), float(omega), float(rcx), float(rcy)))

    def set_mei(self, on):
        self._ck(self.L.lbm2d_set_mei(self.h, int(bool(on))))

    def set_body_force(self, fx):
        self._ck(self.L.lbm2d_set_body_force(self.h, float(fx)))

    def set_thermal(self, use, T_ref=1.0, alpha=0.1666666667, omega_k=1.0, beta=0.0, g_buoyancy=0.0):
        self._ck(self.L.lbm2d_set_thermal(self.h, int(bool(use)), T_ref, alpha, omega_k, beta, g_buoyancy))

    def set_thermal_hook(self, kind, Ta=0.0, Tb=0.0):
        self._ck(self.L.lbm2d_set_thermal_hook(self.h, int(kind), float(Ta), float(Tb)))

    def set_block(self, bx, by):
        self._ck(self.L.lbm2d_set_block(self.h, int(bx), int(by)))

    def set_kernel_variant(self, variant: int):
        """0 (default): fastest kernel the configuration allows (row pipeline;
        else paired nodes, flat node pairs in a batch; else one node per
        thread, which the thermal DDF runs); 1: one node per thread; 2: paired
        nodes per thread; 3: the tile pipeline.  `info().kernel` reports the
        kernel in use (KERNEL_SCALAR / KERNEL_PAIR / KERNEL_ROWS /
        KERNEL_TILES)."""
        self._ck(self.L.lbm2d_set_kernel_variant(self.h, int(variant)))

    def set_wait_limit(self, cycles: int):
        """Limit of the row pipeline's consumer waits in SM cycles (0: the
        default of about one second); a tiny limit exercises the timeout path."""
        self._ck(self.L.lbm2d_set_wait_limit(self.h, int(cycles)))

    # -- state
    def upload_f(self, f):
        a = np.ascontiguousarray(f, np.float64).reshape(-1)
        assert a.size == self.nx * self.ny * 9
        self._ck(self.L.lbm2d_upload_f(self.h, _d(a)))

    def upload_g(self, g):
        a = np.ascontiguousarray(g, np.float64).reshape(-1)
        assert a.size == self.nx * self.ny * 9
        self._ck(self.L.lbm2d_upload_g(self.h, _d(a)))

    def init_uniform(self, rho, u, v):
        self.upload_f(equilibrium_field(self.nx, self.ny, rho, u, v))

    def init_equilibrium(self, rho, u, v, T=1.0):
        """Uniform equilibrium f (and g at temperature T) written on the device."""
        self._ck(self.L.lbm2d_init_equilibrium(self.h, float(rho), float(u), float(v), float(T)))

    def step(self, tau, u_in, n=1):
        self._ck(self.L.lbm2d_step(self.h, float(tau), float(u_in), int(n)))

    def synchronize(self):
        self._ck(self.L.lbm2d_synchronize(self.h))

    def force_sums(self):
        a, b = _D(), _D()
        self._ck(self.L.lbm2d_force_sums(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def force_history(self, n=None):
        cnt = _I(0)
        self._ck(self.L.lbm2d_force_history(self.h, None, None, 0, C.byref(cnt)))
        m = cnt.value if n is None else min(n, cnt.value)
        fx, fy = np.zeros(m), np.zeros(m)
        self._ck(self.L.lbm2d_force_history(self.h, _d(fx), _d(fy), m, C.byref(cnt)))
        return fx, fy

    def force_history_reset(self):
        self._ck(self.L.lbm2d_force_history_reset(self.h))

    @property
    def f(self) -> np.ndarray:
        out = np.empty(self.nx * self.ny * 9, np.float64)
        self._ck(self.L.lbm2d_download_f(self.h, _d(out)))
        return out

    @property
    def g(self) -> np.ndarray:
        out = np.empty(self.nx * self.ny * 9, np.float64)
        self._ck(self.L.lbm2d_download_g(self.h, _d(out)))
        return out

    def force_field(self):
        fx = np.empty(self.nx * self.ny, np.float64)
        fy = np.empty(self.nx * self.ny, np.float64)
        self._ck(self.L.lbm2d_download_force_field(self.h, _d(fx), _d(fy)))
        return fx, fy

    @property
    def fx(self):
        return self.force_field()[0]

    @property
    def fy(self):
        return self.force_field()[1]

    def macros(self, thermal=False):
        n = self.nx * self.ny
        rho, u, v = np.empty(n), np.empty(n), np.empty(n)
        T = np.empty(n) if thermal else None
        self._ck(self.L.lbm2d_download_macros(self.h, _d(rho), _d(u), _d(v), _d(T) if thermal else None))
        return (rho, u, v, T) if thermal else (rho, u, v)

    def set_ibm(self, points, dt=1.0, u_wall=(0.0, 0.0)):
        """Immersed-boundary direct forcing around every step at the (n, 2)
        Lagrangian points (the airfoil driver's loop); an empty array
        removes it."""
        pts = np.ascontiguousarray(points, np.float64).reshape(-1, 2)
        X, Y = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
        self._ibm_n = len(X)
        self._ck(self.L.lbm2d_set_ibm(self.h, _d(X), _d(Y), len(X), float(dt), float(u_wall[0]),
                                      float(u_wall[1])))

    def ibm_lagrangian(self):
        """(U, V, FX, FY) at the points: the values that produced the forcing
        of the last step."""
        out = [np.zeros(self._ibm_n) for _ in range(4)]
        self._ck(self.L.lbm2d_ibm_lagrangian(self.h, *(_d(a) for a in out)))
        return tuple(out)

    def frame_fields(self, ds, sanitize=True, T_wall=0.0):
        """Fields of the reference's frame writers at nodes (i*ds, j*ds),
        computed on the device: dict of (nyd, nxd) arrays rho, u, v, vel,
        omega, T (float64) and obstacle (uint8).  sanitize=True applies the
        JSON writers' NaN / zero-density replacements, False gives the raw
        values the VTK writer prints."""
        d = max(int(ds), 1)  # the library rejects ds < 1
        nxd, nyd = (self.nx + d - 1) // d, (self.ny + d - 1) // d
        out = {k: np.empty(nxd * nyd) for k in ("rho", "u", "v", "vel", "omega", "T")}
        ob = np.empty(nxd * nyd, np.uint8)
        self._ck(self.L.lbm2d_frame_fields(self.h, int(ds), 1 if sanitize else 0, float(T_wall),
                                           *(_d(out[k]) for k in ("rho", "u", "v", "vel", "omega", "T")),
                                           _u8(ob)))
        out["obstacle"] = ob
        return {k: a.reshape(nyd, nxd) for k, a in out.items()}

    def diagnostics(self):
        """(mass, momentum x, momentum y, residual) in FP64 over fluid nodes."""
        m, a, b, r = _D(), _D(), _D(), _D()
        self._ck(self.L.lbm2d_diagnostics(self.h, C.byref(m), C.byref(a), C.byref(b), C.byref(r)))
        return m.value, a.value, b.value, r.value

    @property
    def wall_dist(self):
        out = np.empty(self.nx * self.ny, np.float64)
        self._ck(self.L.lbm2d_download_wall_dist(self.h, _d(out)))
        return out

    def info(self) -> Info:
        i = Info()
        self._ck(self.L.lbm2d_get_info(self.h, C.byref(i)))
        return i

    def set_profiling(self, on: bool):
        self._ck(self.L.lbm2d_set_profiling(self.h, int(bool(on))))

    def profile(self):
        """(summed step-kernel milliseconds, timed launches) since the last call."""
        ms, n = _D(), C.c_longlong()
        self._ck(self.L.lbm2d_profile(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def upload_f_ptr(self, host_ptr: int):
        """Upload populations from a host pointer (e.g. pinned memory)."""
        self._ck(self.L.lbm2d_upload_f(self.h, C.cast(host_ptr, _DP)))

    def download_f_ptr(self, host_ptr: int):
        self._ck(self.L.lbm2d_download_f(self.h, C.cast(host_ptr, _DP)))

    def autotune(self, tau, u_in, steps=20):
        """Pick the fastest launch shape for this solver (state is preserved)."""
        bx, by = _I(), _I()
        self._ck(self.L.lbm2d_autotune(self.h, int(steps), float(tau), float(u_in), C.byref(bx), C.byref(by)))
        return bx.value, by.value

    @property
    def stream(self) -> int:
        return int(self.L.lbm2d_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.L.lbm2d_launch_count(self.h))


class Batch:
    """Many independent solvers stepped by one packed launch per step."""

    def __init__(self, device: int = 0):
        L = lib()
        h = _P()
        rc = L.lbm2d_batch_create(int(device), C.byref(h))
        if rc:
            raise LBMError(rc, "batch create")
        self.L, self.h = L, h
        self.members: list[Solver] = []

    def _ck(self, rc):
        if rc:
            raise LBMError(rc, self.L.lbm2d_batch_last_error(self.h).decode())

    def add(self, solver: Solver, tau: float, u_in: float):
        self._ck(self.L.lbm2d_batch_add(self.h, solver.h, float(tau), float(u_in)))
        self.members.append(solver)

    def remove(self, solver: Solver):
        self._ck(self.L.lbm2d_batch_remove(self.h, solver.h))
        self.members.remove(solver)

    def set_params(self, solver: Solver, tau: float, u_in: float):
        self._ck(self.L.lbm2d_batch_set_params(self.h, solver.h, float(tau), float(u_in)))

    def set_budget(self, solver: Solver, steps: int):
        """The member takes at most `steps` more steps (-1: unlimited)."""
        self._ck(self.L.lbm2d_batch_set_budget(self.h, solver.h, int(steps)))

    def budget(self, solver: Solver) -> int:
        return int(self.L.lbm2d_batch_budget(self.h, solver.h))

    def step(self, n: int = 1):
        self._ck(self.L.lbm2d_batch_step(self.h, int(n)))

    def synchronize(self):
        self._ck(self.L.lbm2d_batch_synchronize(self.h))

    def set_block(self, bx, by):
        self._ck(self.L.lbm2d_batch_set_block(self.h, int(bx), int(by)))

    def autotune(self, steps=10):
        bx, by = _I(), _I()
        self._ck(self.L.lbm2d_batch_autotune(self.h, int(steps), C.byref(bx), C.byref(by)))
        return bx.value, by.value

    @property
    def stream(self) -> int:
        return int(self.L.lbm2d_batch_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.L.lbm2d_batch_launch_count(self.h))

    def __len__(self):
        return int(self.L.lbm2d_batch_size(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm2d_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop: concurrent solves admitted by device-memory footprint and
    stepped together (see include/lbm2d.h, lbm2d_server_*)."""

    def __init__(self, device=0, budget_bytes=64 << 30, max_active=512, steps_per_tick=200, resident=False,
                 fifo=False):
        """resident: step the solves with the device-resident loop
        (LBM2D_SERVE_RESIDENT; steps_per_tick then bounds one launch of the
        loop) instead of host ticks of steps_per_tick batched steps.  fifo
        (ticks): every active solve in every tick, instead of the fewest
        remaining steps first (LBM2D_SERVE_FIFO)."""
        L = lib()
        h = _P()
        rc = L.lbm2d_server_create_ex(int(device), float(budget_bytes), int(max_active), int(steps_per_tick),
                                      (1 if resident else 0) | (2 if fifo else 0), C.byref(h))
        if rc:
            raise LBMError(rc, "server create")
        self.L, self.h = L, h
        self._state = {}  # id -> (f_out, g_out) buffers the server writes at retirement

    def submit(self, nx, ny, geometry, re, steps, storage="fp16", param=0.0, u=0.1, f_init=None,
               keep_state=False) -> int:
        """Queue one solve.  f_init (optional): its initial populations, FP64
        AoS, instead of the geometry's equilibrium start.  keep_state: the
        final populations (and, for the heated cavity, the temperature
        populations) are returned with the result as "f" / "g"."""
        r = Request(int(nx), int(ny), int(geometry), float(re), float(param), float(u), int(steps),
                    STORAGE[storage] if isinstance(storage, str) else int(storage))
        rid = C.c_longlong()
        if f_init is None and not keep_state:
            rc = self.L.lbm2d_server_submit(self.h, C.byref(r), C.byref(rid))
        else:
            n9 = int(nx) * int(ny) * 9
            fi = None if f_init is None else np.ascontiguousarray(f_init, np.float64).reshape(-1)
            assert fi is None or fi.size == n9
            fo = np.full(n9, np.nan) if keep_state else None
            go = np.full(n9, np.nan) if keep_state and int(geometry) == GEOM_HEATED_CAVITY else None
            rc = self.L.lbm2d_server_submit_state(self.h, C.byref(r), None if fi is None else _d(fi),
                                                  None if fo is None else _d(fo), None if go is None else _d(go),
                                                  C.byref(rid))
            if not rc and keep_state:
                self._state[rid.value] = (fo, go)
        if rc:
            raise LBMError(rc, "submit")
        return rid.value

    def wait(self, n_finished, timeout_s=600.0) -> bool:
        return self.L.lbm2d_server_wait(self.h, int(n_finished), float(timeout_s)) == 0

    def results(self) -> list[dict]:
        n = _I()
        self.L.lbm2d_server_results(self.h, None, 0, C.byref(n))
        arr = (Result * max(n.value, 1))()
        self.L.lbm2d_server_results(self.h, arr, n.value, C.byref(n))
        keys = [k for k, _ in Result._fields_]
        out = [{k: getattr(arr[i], k) for k in keys} for i in range(n.value)]
        for x in out:
            if x["id"] in self._state:
                x["f"], x["g"] = self._state[x["id"]]
        return out

    def stats(self) -> dict:
        st = ServerStats()
        self.L.lbm2d_server_stats(self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None):
            self.L.lbm2d_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
