"""Benchmark of the GB300 D2Q9 lattice-Boltzmann step.

Workload (one "step" = one time step over the whole lattice):
  periodic-x channel, 4096 x 4096 nodes, solid rows y=0 and y=NY-1, 64 seeded
  non-overlapping circles (R 8..40), MRT + Smagorinsky/Van Driest LES
  (Cs = 0.1), Re = 1000 on the channel height with u = 0.1, body-force
  driven, momentum-exchange drag/lift reduced every step -- the large-domain
  precision-study configuration, FP32 storage (plain path) and the FP16/BF16
  shifted-deviation storage beside it.

Printed JSON line (rank 0):
  value       whole-job GLUPS of the FP32 step, inputs resident in HBM
  e2e         GLUPS through the public API with host buffers: initial state
              uploaded from pinned host memory, every step followed by the
              driver's drag/lift read-back, final state downloaded
  roofline    step-kernel HBM roofline from CUDA events around each launch
  cpu_baseline the CPU oracle (OpenMP restatement of the reference step) on a
              bounded sample of the same workload on this host's cores

`--impl reference` times the reference's CPU algorithm (the oracle port) on a
bounded sample and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "lbm-2d_gb300"), os.path.join(ROOT, "tests", "golden")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import cases as CS  # noqa: E402  (workload geometry generator)

NX, NY = 4096, 4096
N_CIRCLES, RMIN, RMAX, SEED = 64, 8, 40, 2024
U0, RE, CS_LES = 0.1, 1000.0, 0.1
H_CH = NY - 2  # channel height between the solid rows
NU = U0 * H_CH / RE
TAU = 0.5 + 3.0 * NU
BODY_FORCE = 12.0 * NU * U0 / (H_CH * H_CH)  # plane Poiseuille: u_bulk = a H^2 / (12 nu)


def workload_name(nx, ny):
    return (f"channel {nx}x{ny}, periodic x, solid rows y=0,NY-1, {N_CIRCLES} circles R{RMIN}-{RMAX} "
            f"seed {SEED}, MRT+Smagorinsky/VanDriest Cs={CS_LES}, Re={RE:g} on channel height {H_CH} "
            f"with u={U0} (tau={TAU:.6f}), body force {BODY_FORCE:.3e}")


WORKLOAD = workload_name(NX, NY)

# lbm2d_info.kernel -> (kernel function, description)
KERNEL_NAMES = {0: ("step_kernel", "one node per thread"),
                1: ("step_pair_kernel", "two x-neighbours per thread, packed FP32x2, register pulls"),
                2: ("step_rows_kernel", "row tiles staged by cp.async.bulk into shared memory, persistent grid, "
                                        "packed FP32x2"),
                3: ("step_tiles_kernel", "flat tiles of 512 consecutive nodes staged by cp.async.bulk, persistent "
                                         "grid over one or many instances")}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_record():
    """DRAM bytes per step-kernel launch from one ncu capture of this workload
    (profiles/step_rows_kernel_4096x4096_dram.json, with the command that made it)."""
    p = os.path.join(ROOT, "profiles", "step_rows_kernel_4096x4096_dram.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return None
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed regions."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.rows: list[list[str]] = []
        self.proc = None
        self.active = False
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            if self.active:
                self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_geometry(nx=NX, ny=NY, n_circles=N_CIRCLES):
    mask, circles = CS.channel_circles_mask(nx, ny, n_circles, RMIN, RMAX, SEED)
    return mask, circles


def configure(lbm2d, storage, mask, circles, device=0, nx=NX, ny=NY, les=True):
    s = lbm2d.Solver(nx, ny, lbm2d.RIBS, lbm2d.MRT, les, CS_LES, storage, device)
    s.set_mask(mask)
    cx, cy, r = circles[-1]
    s.set_bb_cylinder(cx, cy, r)  # bb_geom keeps the last placed circle (unused by the periodic case)
    s.set_body_force(BODY_FORCE)
    return s


def time_device(s, torch, steps, warmup):
    """Device time of exactly `steps` steps (CUDA events on the solver's
    stream) as a caller runs them: one multi-step call, which replays a
    captured graph of step pairs.  Then the step kernel's own average time
    from a second pass of the same length with per-kernel events (profiling
    switches the graph off), for the roofline."""
    stream = torch.cuda.ExternalStream(s.stream)
    s.step(TAU, U0, warmup)
    s.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    l0 = s.launches
    e0.record(stream)
    s.step(TAU, U0, steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    launches = s.launches - l0
    ms = e0.elapsed_time(e1)
    s.set_profiling(True)
    s.profile()
    s.step(TAU, U0, steps)
    s.synchronize()
    kms, kn = s.profile()
    s.set_profiling(False)
    s.synchronize()
    return ms, kms / max(kn, 1), launches


def time_e2e(lbm2d, s, torch, steps, f0_pinned, fout_pinned):
    """Public-API run with host buffers: upload, per-step step + drag/lift
    read-back (the drivers' loop, src/main.cpp:103-122), final download."""
    torch.cuda.synchronize()
    l0 = s.launches
    t0 = time.perf_counter()
    s.upload_f_ptr(f0_pinned.data_ptr())
    ta = time.perf_counter()
    for _ in range(steps):
        s.step(TAU, U0, 1)
        s.force_sums()
    tb = time.perf_counter()
    s.download_f_ptr(fout_pinned.data_ptr())
    t1 = time.perf_counter()
    phases = {"upload_ms": (ta - t0) * 1e3, "steps_ms": (tb - ta) * 1e3, "download_ms": (t1 - tb) * 1e3}
    return (t1 - t0) * 1e3, s.launches - l0, phases


def _cpu_impl():
    """Which CPU implementation of the reference step times the CPU legs: the
    reference's own headers compiled here (oracle/_ref, kind "reference")
    when that build exists and loads on this host, else the C restatement
    (kind "port")."""
    from oracle import oracle as O
    if os.path.exists(O.LIB_REF):
        try:
            O.Solver(8, 8, "ref").close()
            return "ref", "reference", "the reference's src/lbm.hpp step compiled by oracle/Makefile (OpenMP)"
        except OSError:
            pass
    if not os.path.exists(O.LIB_ORACLE):
        O.build()
    return "oracle", "port", "oracle/lbm_oracle.c (OpenMP restatement of the reference step)"


def _oracle_channel(size, kind="oracle", ny=None):
    """The channel workload in the oracle: size x size with the circle count
    scaled by area, or (with ny) exactly the nx x ny workload of the GPU runs."""
    from oracle import oracle as O
    if not os.path.exists(O.LIB_ORACLE):
        O.build()
    nx = size
    if ny is None:
        ny = size
        nc = max(1, int(round(N_CIRCLES * (size * size) / (NX * NY))))
    else:
        nc = N_CIRCLES
    mask, _ = CS.channel_circles_mask(nx, ny, nc, RMIN, RMAX, SEED)
    s = O.Solver(nx, ny, kind)
    s.set_case(O.RIBS, O.MRT, True, CS_LES)
    s.obstacle[:] = mask
    s.set_body_force(BODY_FORCE)
    s.init_uniform(1.0, U0, 0.0)
    return s, nc


def cpu_sample(size: int = 1024, budget_s: float = 12.0, max_steps: int = 50):
    """The oracle (OpenMP restatement of the reference step, including its
    per-step wall-distance sweep under LES) on a bounded sample of the
    workload: the same generator and physics at size x size, circles scaled
    by area; steps are timed until about `budget_s` of CPU work."""
    kind, _, _ = _cpu_impl()
    s, nc = _oracle_channel(size, kind)
    s.step(TAU, U0)  # warm-up
    n, t0 = 0, time.perf_counter()
    while n < max_steps and (time.perf_counter() - t0) < budget_s:
        s.step(TAU, U0)
        n += 1
    dt = time.perf_counter() - t0
    s.close()
    return size * size * n / dt / 1e6, dt, nc, n


def _cpu_model():
    """The host CPU's model name and logical core count (lscpu)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        model = next((l.split(":", 1)[1].strip() for l in out.splitlines() if l.startswith("Model name")), "?")
    except Exception:
        model = "?"
    return f"{model}, {os.cpu_count()} logical cores"


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    kind, ckind, what = _cpu_impl()
    # the GPU arm's own workload (nx x ny, the same 64 circles) unless a
    # square sample is asked for; steps stop at the time budget
    if args.ref_size > 0:
        nx = ny = args.ref_size
        s, nc = _oracle_channel(nx, kind)
    else:
        nx, ny = args.nx, args.ny
        s, nc = _oracle_channel(nx, kind, ny)
    same = (nx, ny) == (args.nx, args.ny)
    # a CPU loop needs no warm-up beyond its first touch of the arrays; at the
    # full size one step takes about a minute (the reference's per-step
    # wall-distance sweep), so only a sample warms up
    for _ in range(0 if same else min(args.warmup, 1)):
        s.step(TAU, U0)
    per = []
    t_all = time.perf_counter()
    for _ in range(args.steps):  # each step is one oracle step over the whole sample
        t0 = time.perf_counter()
        s.step(TAU, U0)
        per.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > args.ref_budget:
            break
    s.close()
    dt = float(np.sum(per))
    value = nx * ny * len(per) / dt / 1e9
    size = f"{nx}x{ny}"
    line = {
        "impl": "reference", "metric": "GLUPS (D2Q9 step, lattice updates/s) & %HBM roofline, FP32 vs FP16/BF16 storage",
        "value": value, "unit": "GLUPS", "n_gpus": args.gpus, "steps": len(per), "warmup": args.warmup,
        "ms_per_step": dt / len(per) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.nx, args.ny), "same_config": same,
                   "sample": f"{size} with {nc} circles (same generator and physics), "
                             f"{len(per)} of {args.steps} requested steps within {args.ref_budget:.0f} s"},
        "cpu_baseline": {"value": value, "unit": "GLUPS", "cores": cores, "kind": ckind, "cpu": _cpu_model(),
                         "sample": f"{what}, its per-step wall-distance sweep included, {cores} threads, "
                                   f"{size}, {len(per)} steps"},
        "e2e": {"value": value, "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------- batch / serving
def _c4_instances(n=256, seed=7):
    """256 uneven solves: sides log-uniform in [64, 1024], aspect 1-3, case in
    {cavity, step, cylinder}, Re ~ U[50, 1000] with u = 0.1, 30% heated
    cavities (Pr 0.71, Ra <= 1e5)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        side = int(np.exp(rng.uniform(np.log(64), np.log(1024))))
        aspect = rng.uniform(1.0, 3.0)
        if rng.random() < 0.3:
            out.append(dict(nx=side, ny=side, geometry=4, re=0.0, param=float(10 ** rng.uniform(3, 5))))
            continue
        geom = int(rng.integers(0, 3))
        nx, ny = (side, side) if geom == 0 else (int(side * aspect), side)
        out.append(dict(nx=max(nx, 16), ny=max(ny, 16), geometry=geom, re=float(rng.uniform(50, 1000)), param=0.0))
    return out


def _c5_requests(n, seed=11):
    """Serving stream: grids 128x64 .. 2048x768 (log-uniform), geometry in
    {cavity, step h=H/3, cylinder D=H/5, side-by-side S/D in [2,5]},
    Re ~ U[50, 2000], budgets log-uniform in [1k, 50k] steps."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        t = rng.uniform(0, 1)
        nx = int(np.exp(np.log(128) + t * (np.log(2048) - np.log(128))))
        ny = int(np.exp(np.log(64) + t * (np.log(768) - np.log(64))))
        geom = int(rng.integers(0, 4))
        if geom == 0:
            ny = nx = max(64, int(np.sqrt(nx * ny)))
        out.append(dict(nx=nx, ny=ny, geometry=geom, re=float(rng.uniform(50, 2000)),
                        param=float(rng.uniform(2, 5)) if geom == 3 else 0.0,
                        steps=int(np.exp(rng.uniform(np.log(1000), np.log(50000))))))
    return out


def run_serve(args):
    import lbm2d
    lbm2d.build(quiet=True)
    print(json.dumps(serve_block(args, lbm2d)), flush=True)
    return 0


def serve_block(args, lbm2d):
    """Poisson arrivals (rate --rate) of --requests solves through the serving
    loop, against the same requests solved one at a time with the plain
    per-solve API (lbm2d_step) on the same GPU."""
    reqs = _c5_requests(args.requests)
    scale = args.budget_scale  # scales every step budget (bounded run time)
    for r in reqs:
        r["steps"] = max(100, int(r["steps"] * scale))
    rng = np.random.default_rng(5)
    gaps = rng.exponential(1.0 / args.rate, len(reqs))
    storage = args.serve_storage

    def leg(resident, fifo=False):
        # resident: the device loop (steps_per_tick bounds one launch of it);
        # else host ticks of args.tick batched steps, the fewest remaining
        # steps first (fifo: every active solve in every tick)
        srv = lbm2d.Server(0, budget_bytes=args.serve_budget_gb * (1 << 30), max_active=args.max_active,
                           steps_per_tick=args.resident_launch if resident else args.tick, resident=resident,
                           fifo=fifo)
        t0 = time.perf_counter()
        next_t = t0
        for r, gap in zip(reqs, gaps):
            next_t += gap
            while time.perf_counter() < next_t:
                time.sleep(min(0.001, max(0.0, next_t - time.perf_counter())))
            srv.submit(r["nx"], r["ny"], r["geometry"], r["re"], r["steps"], storage, r["param"])
        srv.wait(len(reqs), timeout_s=3600)
        res = srv.results()
        st = srv.stats()
        srv.close()
        lat = np.array([x["t_done"] - x["t_submit"] for x in res])
        lu = sum(x["steps"] * x["nodes"] for x in res)
        span = max(x["t_done"] for x in res) - min(x["t_submit"] for x in res)
        status = {}
        for x in res:
            status[str(x["status"])] = status.get(str(x["status"]), 0) + 1
        out = {"loop": "resident" if resident else ("ticks, every solve each tick" if fifo else
                                                     "ticks, fewest remaining steps first"),
               "requests": len(res), "failed": int(sum(1 for x in res if x["status"] != 0)), "status": status,
               "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
               "mean_s": float(lat.mean()), "makespan_s": span, "glups": lu / span / 1e9,
               "busy_glups": st["lattice_updates"] / max(st["busy_s"], 1e-9) / 1e9, "lattice_updates": lu,
               "setup_s": st["setup_s"], "gpu_s": st["gpu_s"],
               "stepping_thread_s": {k: st[k] for k in ("call_s", "wait_s", "retire_s", "join_s")},
               "gpu_glups": st["lattice_updates"] / max(st["gpu_s"], 1e-9) / 1e9}
        if resident:
            out["launches"] = st["ticks"]
        else:
            out["ticks"] = st["ticks"]
            out["mean_solves_per_tick"] = st["member_ticks"] / max(st["ticks"], 1)
        return out

    # the tick loop is the headline (the faster of the two on this mix); the
    # device-resident loop is measured beside it
    serve = leg(False)
    serve_fifo = leg(False, fifo=True) if not args.no_resident_leg else None
    serve_resident = leg(True) if not args.no_resident_leg else None
    # --- sequential plain solves, FIFO, same arrival times:
    #   "dropin": the reference drivers' loop through the per-solve API, one
    #             lbm2d_step call per time step followed by the drag/lift
    #             read-back (src/main.cpp:103-122);
    #   "bulk":   one lbm2d_step call for the whole budget, no per-step read-back.
    seq = {}
    if not args.no_sequential:
        import torch  # noqa: F401  (CUDA context for timing parity)
        arrivals = np.cumsum(gaps)
        for mode in ("dropin", "bulk"):
            clock = 0.0
            lat_s = []
            lu_s = 0
            wall0 = time.perf_counter()
            failed = 0
            for r, at in zip(reqs, arrivals):
                start = max(clock, at)
                ts = time.perf_counter()
                s = _plain_solver(lbm2d, r, storage)
                if mode == "bulk":
                    s.step(s._tau, s._ubc, r["steps"])
                else:
                    for _ in range(r["steps"]):
                        s.step(s._tau, s._ubc, 1)
                        s.force_sums()
                try:
                    s.synchronize()
                except lbm2d.LBMError:  # diverged (non-finite density), as the reference would
                    failed += 1
                s.close()
                dt = time.perf_counter() - ts
                clock = start + dt
                lat_s.append(clock - at)
                lu_s += r["steps"] * r["nx"] * r["ny"]
            busy = time.perf_counter() - wall0
            lat_s = np.array(lat_s)
            seq[mode] = {"p50_s": float(np.percentile(lat_s, 50)), "p99_s": float(np.percentile(lat_s, 99)),
                         "failed": failed, "makespan_s": clock, "glups": lu_s / clock / 1e9,
                         "busy_glups": lu_s / busy / 1e9}
        seq["dropin"]["note"] = ("same requests and arrival times solved one at a time, FIFO, through the "
                                 "per-solve API as the reference drivers step: one lbm2d_step call per time step "
                                 "+ drag/lift read-back")
        seq["bulk"]["note"] = "same, but one lbm2d_step call for each request's whole budget"
    line = {"metric": "serving: p50/p99 time-to-solution and aggregate GLUPS", "unit": "GLUPS",
            "value": serve["glups"], "p50_s": serve["p50_s"], "p99_s": serve["p99_s"], "glups": serve["glups"],
            "budget_scale": scale, "serve": serve, "serve_fifo": serve_fifo, "serve_resident": serve_resident,
            "sequential": seq or None,
            "speedup_vs_sequential_dropin": (serve["glups"] / seq["dropin"]["glups"]) if seq else None,
            "speedup_vs_sequential_bulk": (serve["glups"] / seq["bulk"]["glups"]) if seq else None,
            "config": {"workload": f"{len(reqs)} requests, Poisson {args.rate}/s, grids 128x64..2048x768, "
                                   f"{{cavity, step, cylinder, side-by-side}}, Re 50-2000, budgets 1k-50k x {scale}",
                       "storage": storage, "loop": "ticks, fewest remaining steps first (16 Mi nodes per tick)",
                       "resident_launch": args.resident_launch,
                       "tick": args.tick, "budget_gb": args.serve_budget_gb}}
    return line


def _plain_solver(lbm2d, r, storage):
    """One request set up through the plain per-solve API, as the serving loop
    sets it up (same geometry rules)."""
    nx, ny, geom = r["nx"], r["ny"], r["geometry"]
    u = 0.1
    mask = np.zeros(nx * ny, np.uint8)
    L = lbm2d.lib()
    bb = None
    thermal = geom == 4
    if geom == 0:
        case, Lc = lbm2d.CAVITY, nx
        L.lbm2d_mask_walls(nx, ny, lbm2d._u8(mask))
    elif geom == 1:
        case = lbm2d.STEP
        hs = ny // 3
        m = mask.reshape(ny, nx)
        m[0, :] = 1
        m[ny - 1, :] = 1
        m[:hs, : nx // 4] = 1
        Lc = 2.0 * (ny - 1 - hs)
    elif geom == 2:
        case, Lc = lbm2d.CYLINDER, ny / 5.0
        bb = (nx // 4, ny // 2 + 1, ny // 10)
        L.lbm2d_mask_cylinder(nx, ny, lbm2d._u8(mask), *bb)
    elif geom == 3:
        case = lbm2d.SIDE_BY_SIDE
        rad = ny // 10
        D = 2 * rad
        sp = int((r["param"] or 3.0) * D)
        cy1 = ny // 2 - sp // 2
        L.lbm2d_mask_cylinder(nx, ny, lbm2d._u8(mask), nx // 4, cy1, rad)
        L.lbm2d_mask_cylinder(nx, ny, lbm2d._u8(mask), nx // 4, cy1 + sp, rad)
        bb = (nx // 4, cy1 + sp, rad)
        Lc = D
    else:
        case = lbm2d.CYLINDER
        m = mask.reshape(ny, nx)
        m[:, 0] = m[:, -1] = 1
        m[0, :] = m[-1, :] = 1
        Lc = None
    tau = 0.8 if thermal else 0.5 + 3.0 * (u * Lc / r["re"])
    s = lbm2d.Solver(nx, ny, case, lbm2d.MRT, tau < 0.55, 0.12, storage)
    s.set_mask(mask)
    if bb:
        s.set_bb_cylinder(*bb)
    ubc = u
    if thermal:
        Pr, Th, Tc = 0.71, 1.5, 0.5
        nu = (tau - 0.5) / 3.0
        alpha = nu / Pr
        gb = (r["param"] or 1e4) * nu * alpha / ((Th - Tc) * ny ** 3)
        s.set_thermal(True, 1.0, alpha, 1.0 / (0.5 + 3.0 * alpha), 0.001, -gb / 0.001)
        s.set_thermal_hook(lbm2d.HOOK_HEATED_CAVITY, Th, Tc)
        ubc = 0.0
    s.init_equilibrium(1.0, u if geom in (2, 3) else 0.0, 0.0, 1.0)
    s._tau, s._ubc = tau, ubc
    return s


def run_batch(args):
    import lbm2d
    lbm2d.build(quiet=True)
    print(json.dumps(batch_block(args, lbm2d, args.batch_storage, args.steps)), flush=True)
    return 0


def batch_block(args, lbm2d, storage, steps):
    """256 uneven solves stepped together (one packed launch per step per
    storage group) against the same solves stepped one after another, each
    in one whole-budget call."""
    import torch
    inst = _c4_instances(args.instances)
    nodes = sum(r["nx"] * r["ny"] for r in inst)

    def diverged(solvers):
        n = 0
        for s in solvers:
            try:
                s.synchronize()
            except lbm2d.LBMError as ex:  # a solve that diverges does so in both legs alike
                if ex.code != 4:
                    raise
                n += 1
        return n

    # sequential: each solver alone, one after the other, from the same start
    solvers = [_plain_solver(lbm2d, r, storage) for r in inst]
    for s in solvers:
        s.step(s._tau, s._ubc, 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in solvers:
        s.step(s._tau, s._ubc, steps)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    nan_seq = diverged(solvers)
    for s in solvers:
        s.close()
    # batched: fresh solvers from the same start
    solvers = [_plain_solver(lbm2d, r, storage) for r in inst]
    b = lbm2d.Batch()
    for s in solvers:
        b.add(s, s._tau, s._ubc)
    if args.autotune:
        bx, by = b.autotune(5)
    b.step(2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    l0 = b.launches
    b.step(steps)
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t0
    nan = diverged(solvers)
    bytes_lu = sum(r["nx"] * r["ny"] * 18 * lbm2d.BYTES_PER_POP[storage] * (2 if r["geometry"] == 4 else 1)
                   for r in inst) / nodes
    peak, peak_kind = peaks()
    glups = nodes * steps / t_bat / 1e9
    line = {"metric": "batched uneven solves: aggregate GLUPS", "unit": "GLUPS",
            "value": glups, "glups": glups, "sequential_glups": nodes * steps / t_seq / 1e9,
            "speedup_vs_sequential": t_seq / t_bat, "steps": steps, "instances": len(inst), "nodes": nodes,
            "batch_launches": b.launches - l0, "diverged": nan, "diverged_sequential": nan_seq,
            "kernels": sorted({KERNEL_NAMES[s.info().kernel][0] for s in solvers}),
            "thermal_instances": sum(1 for r in inst if r["geometry"] == 4),
            "alg_bytes_per_update": bytes_lu, "roofline_frac": glups * bytes_lu / peak, "peak_kind": peak_kind,
            "config": {"workload": "256 uneven cavity/step/cylinder solves, sides log-uniform 64-1024, aspect 1-3, "
                                   "Re U[50,1000], u=0.1, 30% heated cavities (Pr 0.71, Ra<=1e5)",
                       "storage": storage,
                       "sequential": "the same solves one after another, one lbm2d_step call per whole budget"}}
    b.close()
    for s in solvers:
        s.close()
    return line


def thermal_block(lbm2d, torch, n=4096, steps=200, storages=("fp32", "fp16")):
    """The thermal double-distribution step on its own: the heated-cavity
    driver's set-up (src/thermal_cavity.cpp: walls all round, hot left and cold
    right columns, adiabatic top and bottom rows, Boussinesq buoyancy at
    Ra = 1e5, Pr 0.71, tau 0.8) on an n x n grid, device-timed over `steps`
    steps of one multi-step call.  Bytes per update count both population
    sets (FP32: 144 B, FP16: 72 B)."""
    peak, peak_kind = peaks()
    out = {}
    for st in storages:
        r = dict(nx=n, ny=n, geometry=4, re=0.0, param=1e5)
        s = _plain_solver(lbm2d, r, st)
        stream = torch.cuda.ExternalStream(s.stream)
        s.step(s._tau, s._ubc, 20)
        s.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = s.launches
        e0.record(stream)
        s.step(s._tau, s._ubc, steps)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        launches = s.launches - l0
        diverged = False
        try:
            s.synchronize()
        except lbm2d.LBMError:
            diverged = True
        kernel = KERNEL_NAMES[s.info().kernel][0]
        if kernel == "step_kernel" and st != "fp64":
            kernel = "step_th_kernel"  # the thermal one-node kernel at six blocks per SM
        s.close()
        bpu = 2 * 2 * 9 * lbm2d.BYTES_PER_POP[st]
        glups = n * n * steps / (ms * 1e-3) / 1e9
        out[st] = {"glups": glups, "ms_per_step": ms / steps, "bytes_per_update": bpu,
                   "achieved_gbs": glups * bpu, "roofline_frac": glups * bpu / peak, "kernel": kernel,
                   "launches_per_step": launches / steps, "diverged": diverged}
    return {"workload": f"heated cavity {n}x{n}, Ra 1e5, Pr 0.71, tau 0.8 (src/thermal_cavity.cpp set-up)",
            "steps": steps, "peak_gbs": peak, "peak_kind": peak_kind, "results": out}


def run_frame(args):
    """Frame export on the channel workload: the JSON frame's fields
    (downsampled by NX/100, as the reference's writer does) and the VTK
    writer's full-resolution fields computed on the device, against what the
    mirror-based writer needs first: the full FP64 state on the host."""
    import lbm2d
    lbm2d.build(quiet=True)
    nx, ny = args.nx, args.ny
    mask, circles = make_geometry(nx, ny)
    s = configure(lbm2d, "fp32", mask, circles, 0, nx, ny, True)
    s.init_equilibrium(1.0, U0, 0.0)
    s.step(TAU, U0, 100)
    s.synchronize()
    ds = max(1, nx // 100)

    def med(fn, reps):
        fn()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3

    frame_ms = med(lambda: s.frame_fields(ds), 20)
    vtk_ms = med(lambda: s.frame_fields(1, sanitize=False), 5)
    host_ms = med(lambda: s.f, 3)
    line = {"metric": "frame export: device fields vs host-mirror download", "unit": "ms",
            "json_frame_device_ms": frame_ms, "vtk_fields_device_ms": vtk_ms, "state_download_ms": host_ms,
            "json_frame_speedup": host_ms / frame_ms, "frame_points": ((nx + ds - 1) // ds) * ((ny + ds - 1) // ds),
            "config": {"workload": workload_name(nx, ny), "storage": "fp32", "ds": ds}}
    s.close()
    print(json.dumps(line), flush=True)
    return 0


def _airfoil_solver(lbm2d, nx, ny, storage, aoa=8.0, re=100.0, spacing=1.5, ibm=True):
    """The airfoil driver's set-up (src/airfoil_ibm.cpp): NACA 2412 at
    (NX/4, NY/2), chord NY/3, obstacle by point-in-polygon, uniform inflow at
    the angle of attack; Lagrangian points every `spacing` cells."""
    import math
    poly = lbm2d.transform_points(lbm2d.naca_coords(2412, 100), nx / 4, ny / 2, ny / 3.0, aoa)
    mask = np.zeros(nx * ny, np.uint8)
    flat = np.ascontiguousarray(poly.reshape(-1))
    lbm2d.lib().lbm2d_mask_polygon(nx, ny, lbm2d._u8(mask), lbm2d._d(flat), len(poly))
    s = lbm2d.Solver(nx, ny, lbm2d.CYLINDER, lbm2d.MRT, False, 0.12, storage)
    s.set_mask(mask)
    a = aoa * math.pi / 180.0
    s.upload_f(lbm2d.equilibrium_field(nx, ny, 1.0, 0.1 * math.cos(a), 0.1 * math.sin(a)))
    pts = lbm2d.ibm_points_from_polygon(poly, spacing)
    if ibm:
        s.set_ibm(pts)
    tau = 0.5 + 3.0 * 0.1 * (ny / 5.0) / re
    return s, tau, pts, mask, poly


def run_ibm(args):
    """Immersed-boundary airfoil (the reference's airfoil driver loop on the
    device): step throughput with and without the boundary attached, and the
    reference loop on the host cores (oracle restatement) for a bounded
    sample."""
    import torch

    import lbm2d
    lbm2d.build(quiet=True)
    out = {}
    # default: the driver's grid and a large one; --nx/--ny pick one size and
    # --steps/--warmup its step counts (a short case for profiling)
    custom = (args.nx, args.ny) != (NX, NY)
    sizes = [(args.nx, args.ny)] if custom else [(800, 300), (4096, 1536)]
    for nx, ny in sizes:
        row = {}
        for label, ibm in (("plain", False), ("ibm", True)):
            s, tau, pts, _, _ = _airfoil_solver(lbm2d, nx, ny, "fp32", ibm=ibm)
            stream = torch.cuda.ExternalStream(s.stream)
            s.step(tau, 0.1, args.warmup if custom else 20)
            s.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            steps = args.steps if custom else (2000 if nx * ny < 1 << 20 else 500)
            l0 = s.launches
            e0.record(stream)
            s.step(tau, 0.1, steps)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            diverged = False
            try:
                s.synchronize()
            except lbm2d.LBMError:
                diverged = True
            row[label] = {"ms_per_step": ms, "glups": nx * ny / ms / 1e6, "launches_per_step": (s.launches - l0) / steps,
                          "diverged": diverged}
            if ibm:
                row["points"] = len(pts)
            s.close()
        row["ibm_overhead"] = row["ibm"]["ms_per_step"] / row["plain"]["ms_per_step"]
        out[f"{nx}x{ny}"] = row
    # the reference loop on the host cores: oracle restatement, 800x300
    cpu = None
    if not args.no_cpu:
        sys.path.insert(0, ROOT)
        from oracle import oracle as O
        if not os.path.exists(O.LIB_ORACLE):
            O.build()
        nx, ny = 800, 300
        s, tau, pts, mask, poly = _airfoil_solver(lbm2d, nx, ny, "fp32", ibm=False)
        s.close()
        o = O.Solver(nx, ny, "oracle")
        o.set_case(O.CYLINDER)
        o.obstacle[:] = mask
        o.f[:] = lbm2d.equilibrium_field(nx, ny, 1.0, 0.1 * np.cos(np.radians(8.0)), 0.1 * np.sin(np.radians(8.0)))
        o.ibm_from_polygon(poly, 1.5)
        o.ibm_step(tau, 0.1, 2)
        t0 = time.perf_counter()
        n = 0
        while time.perf_counter() - t0 < 10.0 and n < 400:
            o.ibm_step(tau, 0.1)
            n += 1
        dt = time.perf_counter() - t0
        o.close()
        cpu = {"value": nx * ny * n / dt / 1e9, "unit": "GLUPS", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{n} immersed-boundary iterations of the airfoil loop at 800x300 (oracle restatement, "
                         f"OpenMP step)"}
    line = {"metric": "immersed-boundary airfoil: step throughput with the boundary's forcing", "unit": "GLUPS",
            "results": out, "cpu_baseline": cpu,
            "config": {"workload": "NACA 2412 airfoil, chord NY/3 at (NX/4, NY/2), AoA 8 deg, Re 100 on NY/5, "
                                   "u=0.1, Lagrangian spacing 1.5, FP32 storage", "storage": "fp32"}}
    print(json.dumps(line), flush=True)
    return 0


def run_precision(args):
    import lbm2d
    lbm2d.build(quiet=True)
    print(json.dumps(precision_block(lbm2d, args.nx, args.ny, args.steps)), flush=True)
    return 0


def precision_block(lbm2d, nx, ny, steps):
    """Error of FP32 / FP16 / BF16 storage against an FP64 run of the same
    kernel on the channel workload: relative L2 of the velocity field over
    fluid nodes and relative error of the mean drag over the second half of
    the run."""
    mask, circles = make_geometry(nx, ny)
    fluid = mask == 0
    out = {}
    ref = None
    for st in ("fp64", "fp32", "fp16", "bf16"):
        s = configure(lbm2d, st, mask, circles, 0, nx, ny, True)
        s.init_equilibrium(1.0, U0, 0.0)
        s.step(TAU, U0, steps)
        s.synchronize()
        rho, u, v = s.macros()
        fx, fy = s.force_history()
        s.close()
        if ref is None:
            ref = (u, v, fx, fy)
            out[st] = {"steps": steps}
            continue
        du = np.sqrt(np.sum((u - ref[0])[fluid] ** 2 + (v - ref[1])[fluid] ** 2) /
                     np.sum(ref[0][fluid] ** 2 + ref[1][fluid] ** 2))
        drag_ref = float(np.mean(ref[2][steps // 2:]))
        drag = float(np.mean(fx[steps // 2:]))
        out[st] = {"velocity_rel_l2_vs_fp64": float(du), "drag_rel_err_vs_fp64": abs(drag - drag_ref) / abs(drag_ref),
                   "drag": drag, "drag_fp64": drag_ref}
    return {"metric": "storage precision vs FP64 (same kernel)", "config": {"workload": workload_name(nx, ny),
            "steps": steps}, "results": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--ny", type=int, default=NY)
    ap.add_argument("--storages", default="fp32,fp16,bf16")
    ap.add_argument("--plain", default="fp32,fp16", help="storages also timed without LES (plain MRT)")
    ap.add_argument("--variant", type=int, default=0, help="step kernel: 0 paired nodes per thread, 1 one node")
    ap.add_argument("--cpu-size", type=int, default=1024)
    ap.add_argument("--ref-budget", type=float, default=120.0, help="seconds cap of the reference arm")
    ap.add_argument("--ref-size", type=int, default=0,
                    help="reference arm on a size x size sample (0: the GPU arm's own nx x ny workload)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end run (default: --steps)")
    ap.add_argument("--mode", default="step",
                    choices=["step", "batch", "serve", "precision", "frame", "ibm", "thermal"])
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--batch-storage", default="fp32")
    ap.add_argument("--autotune", action="store_true")
    ap.add_argument("--requests", type=int, default=200)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--budget-scale", type=float, default=1.0)
    ap.add_argument("--serve-storage", default="fp16")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    ap.add_argument("--max-active", type=int, default=512)
    ap.add_argument("--tick", type=int, default=200)
    ap.add_argument("--resident-launch", type=int, default=1000,
                    help="serving: iterations of one launch of the resident loop")
    ap.add_argument("--no-resident-leg", action="store_true",
                    help="serving: skip the comparison legs (every solve each tick; the device-resident loop)")
    ap.add_argument("--no-sequential", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the precision, thermal, batch and serving blocks of the default line")
    ap.add_argument("--precision-steps", type=int, default=1000)
    ap.add_argument("--batch-steps", type=int, default=5000)
    ap.add_argument("--thermal-n", type=int, default=4096)
    ap.add_argument("--thermal-steps", type=int, default=200)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "batch":
        return run_batch(args)
    if args.mode == "serve":
        return run_serve(args)
    if args.mode == "precision":
        return run_precision(args)
    if args.mode == "frame":
        return run_frame(args)
    if args.mode == "ibm":
        return run_ibm(args)
    if args.mode == "thermal":
        import torch

        import lbm2d
        lbm2d.build(quiet=True)
        print(json.dumps(thermal_block(lbm2d, torch, args.thermal_n, args.thermal_steps)), flush=True)
        return 0

    import torch

    import lbm2d
    lbm2d.build(quiet=True)
    from lbm2d.replicas import Replicas
    reps = Replicas()  # independent replicas, one per GPU: no data-path collective
    rank, world, local = reps.rank, reps.size, reps.local
    torch.cuda.set_device(local)

    nx, ny = args.nx, args.ny
    storages = [x for x in args.storages.split(",") if x]
    runs = [(st, st, True) for st in storages] + [(st + "_plain", st, False) for st in args.plain.split(",") if st]
    mask, circles = make_geometry(nx, ny)
    f0 = lbm2d.equilibrium_field(nx, ny, 1.0, U0, 0.0)
    clocks = ClockSampler(local)
    clocks.start()
    results = {}
    for label, storage, les in runs:
        s = configure(lbm2d, storage, mask, circles, local, nx, ny, les)
        s.set_kernel_variant(args.variant)
        s.upload_f(f0)
        reps.barrier()
        clocks.active = True
        try:
            ms, kms, launches = time_device(s, torch, args.steps, args.warmup)
            nan = False
        except lbm2d.LBMError as ex:  # a diverged run is reported, not timed
            if ex.code != 4:
                raise
            ms, kms, launches, nan = float("nan"), float("nan"), 0, True
        clocks.active = False
        ms = reps.max(ms)
        info = s.info()
        results[label] = dict(ms=ms, kernel_ms=kms, launches=launches, nan=nan, kernel=info.kernel,
                                bytes_per_update=info.bytes_per_update, boundary=info.n_boundary_nodes,
                                force_nodes=info.n_force_nodes, block=(info.block_x, info.block_y))
        if label == storages[0] and not nan:
            results[label]["force"] = s.force_sums()
        if label == storages[0] and not args.no_e2e:
            # end-to-end through the public API with host buffers
            e2e_steps = args.e2e_steps or args.steps
            pin = torch.empty(nx * ny * 9, dtype=torch.float64, pin_memory=True)
            pin.numpy()[:] = f0
            pout = torch.empty(nx * ny * 9, dtype=torch.float64, pin_memory=True)
            s.upload_f(f0)
            s.step(TAU, U0, args.warmup)
            s.synchronize()
            reps.barrier()
            clocks.active = True
            e2e_ms, e2e_launches, phases = time_e2e(lbm2d, s, torch, e2e_steps, pin, pout)
            clocks.active = False
            results["e2e"] = dict(ms=reps.max(e2e_ms), steps=e2e_steps, launches=e2e_launches, phases=phases)
            del pin, pout
        s.close()
    clocks.stop()

    if rank != 0:
        reps.close()
        return 0
    nodes = nx * ny
    peak, peak_kind = peaks()
    main_st = storages[0]
    r0 = results[main_st]
    bpu = 2 * 9 * lbm2d.BYTES_PER_POP[main_st]
    value = world * nodes * args.steps / (r0["ms"] * 1e-3) / 1e9
    alg_bytes = nodes * float(bpu)  # populations read once + written once per lattice update

    def kernel_time(r):
        # A timed step that is exactly one step-kernel launch bounds that
        # kernel's duration from above by the timed region's time per step;
        # otherwise the profiled pass's per-kernel events give it.
        if r["launches"] == args.steps:
            return r["ms"] / args.steps, "timed region, one launch per step"
        return r["kernel_ms"], "profiled pass, per-kernel events"

    k0, k0_src = kernel_time(r0)
    achieved = alg_bytes / (k0 * 1e-3) / 1e9
    tr = traffic_record()
    traffic = None
    if tr and main_st in tr and tr.get("nodes") and KERNEL_NAMES[r0["kernel"]][0] == tr.get("kernel"):
        # bytes per launch scale with the nodes of the launch
        traffic = float(tr[main_st]["dram_bytes_per_launch"]) * nodes / float(tr["nodes"])
    prec = {}
    for label, st, les in runs[1:]:
        r = results[label]
        g = world * nodes * args.steps / (r["ms"] * 1e-3) / 1e9
        b = 2 * 9 * lbm2d.BYTES_PER_POP[st]
        kt, _ = kernel_time(r)
        kach = nodes * b / (kt * 1e-3) / 1e9
        prec[label] = {"glups": g, "vs_" + main_st: g / value, "kernel_ms": kt, "les": les,
                       "kernel": KERNEL_NAMES[r["kernel"]][0],
                       "roofline_frac": kach / peak, "bytes_per_update": b, "diverged": r["nan"]}
    e2e = None
    if "e2e" in results:
        e = results["e2e"]
        e2e = {"value": world * nodes * e["steps"] / (e["ms"] * 1e-3) / 1e9, "unit": "GLUPS",
               "h2d_bytes_per_step": nodes * 9 * 8 / e["steps"], "d2h_bytes_per_step": 16 + nodes * 9 * 8 / e["steps"],
               "steps": e["steps"], "launches": e["launches"], "phases": e["phases"],
               "note": "initial state H2D from pinned memory + per step (step, drag/lift D2H) + final state D2H"}
    cpu = None
    if not args.no_cpu:
        try:
            cores = os.cpu_count() or 1
            _, ckind, what = _cpu_impl()
            mlups, dt, nc, n = cpu_sample(args.cpu_size)
            cpu = {"value": mlups / 1e3, "unit": "GLUPS", "cores": cores, "kind": ckind, "cpu": _cpu_model(),
                   "sample": f"{what}, per-step wall-distance sweep included, {cores} threads, same generator "
                             f"and physics at {args.cpu_size}x{args.cpu_size} with {nc} circles, {n} steps in "
                             f"{dt:.1f} s"}
        except Exception as ex:  # the CPU leg never blocks the GPU line
            cpu = {"value": None, "unit": "GLUPS", "cores": os.cpu_count(), "kind": None,
                   "sample": f"failed: {ex}"}
    line = {
        "metric": "GLUPS (D2Q9 step, lattice updates/s) & %HBM roofline, FP32 vs FP16/BF16 storage",
        "value": value, "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r0["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp32": "f32", "fp64": "f64"}.get(main_st, "f32"), "data": "synthetic",
        "config": {"workload": workload_name(nx, ny), "nx": nx, "ny": ny, "storage": main_st, "tau": TAU,
                   "body_force_x": BODY_FORCE, "l2": "inputs larger than L2 (populations >= 129 MB, no flush)",
                   "parallelism": "replicas" if world > 1 else "single GPU", "block": list(r0["block"]),
                   "boundary_nodes": r0["boundary"], "force_nodes": r0["force_nodes"], "diverged": r0["nan"],
                   "kernel_variant": KERNEL_NAMES[r0["kernel"]][1]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                     "kernel_ms": k0, "kernel_ms_source": k0_src, "kernel_ms_profiled": r0["kernel_ms"],
                     "kernel": KERNEL_NAMES[r0["kernel"]][0]},
        "precision": prec,
        "e2e": e2e,
        "gpu_launches": r0["launches"],
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "drag_lift": r0.get("force"),
    }
    if world == 1 and not args.no_extras:
        # the other rows of the metric, on the same GPU after the timed step:
        # storage error against FP64, the thermal step, the C4 batch and the
        # C5 serving stream
        def guarded(fn):  # a failing block is reported, never blocks the line
            try:
                return fn()
            except Exception as ex:
                return {"error": f"{type(ex).__name__}: {ex}"}

        pe = guarded(lambda: precision_block(lbm2d, nx, ny, args.precision_steps))
        line["precision_vs_fp64"] = pe
        for st, res in pe.get("results", {}).items():
            if st in prec:
                prec[st].update({k: res[k] for k in ("velocity_rel_l2_vs_fp64", "drag_rel_err_vs_fp64")})
        line["thermal"] = guarded(lambda: thermal_block(lbm2d, torch, args.thermal_n, args.thermal_steps))
        line["batch"] = {st: guarded(lambda st=st: batch_block(args, lbm2d, st, args.batch_steps))
                         for st in ("fp32", "fp16")}
        line["serving"] = guarded(lambda: serve_block(args, lbm2d))
    print(json.dumps(line), flush=True)
    reps.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
