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


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_record():
    p = os.path.join(ROOT, "profiles", "traffic.json")
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
    """Device time of exactly `steps` steps (CUDA events on the solver's stream)."""
    stream = torch.cuda.ExternalStream(s.stream)
    s.step(TAU, U0, warmup)
    s.synchronize()
    s.set_profiling(True)
    s.profile()
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
    kms, kn = s.profile()
    s.set_profiling(False)
    s.synchronize()
    return e0.elapsed_time(e1), kms / max(kn, 1), launches


def time_e2e(lbm2d, s, torch, steps, f0_pinned, fout_pinned):
    """Public-API run with host buffers: upload, per-step step + drag/lift
    read-back (the drivers' loop, src/main.cpp:103-122), final download."""
    torch.cuda.synchronize()
    l0 = s.launches
    t0 = time.perf_counter()
    s.upload_f_ptr(f0_pinned.data_ptr())
    for _ in range(steps):
        s.step(TAU, U0, 1)
        s.force_sums()
    s.download_f_ptr(fout_pinned.data_ptr())
    t1 = time.perf_counter()
    return (t1 - t0) * 1e3, s.launches - l0


def _oracle_channel(size):
    from oracle import oracle as O
    if not os.path.exists(O.LIB_ORACLE):
        O.build()
    nc = max(1, int(round(N_CIRCLES * (size * size) / (NX * NY))))
    mask, _ = CS.channel_circles_mask(size, size, nc, RMIN, RMAX, SEED)
    s = O.Solver(size, size)
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
    s, nc = _oracle_channel(size)
    s.step(TAU, U0)  # warm-up
    n, t0 = 0, time.perf_counter()
    while n < max_steps and (time.perf_counter() - t0) < budget_s:
        s.step(TAU, U0)
        n += 1
    dt = time.perf_counter() - t0
    s.close()
    return size * size * n / dt / 1e6, dt, nc, n


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    size = args.cpu_size
    s, nc = _oracle_channel(size)
    for _ in range(min(args.warmup, 1)):
        s.step(TAU, U0)
    per = []
    t_all = time.perf_counter()
    for _ in range(args.steps):  # each step is one oracle step over the size x size sample
        t0 = time.perf_counter()
        s.step(TAU, U0)
        per.append(time.perf_counter() - t0)
        if time.perf_counter() - t_all > args.ref_budget:
            break
    s.close()
    dt = float(np.sum(per))
    value = size * size * len(per) / dt / 1e9
    line = {
        "impl": "reference", "metric": "GLUPS (D2Q9 step, lattice updates/s) & %HBM roofline, FP32 vs FP16/BF16 storage",
        "value": value, "unit": "GLUPS", "n_gpus": args.gpus, "steps": len(per), "warmup": args.warmup,
        "ms_per_step": dt / len(per) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(args.nx, args.ny),
                   "sample": f"{size}x{size} with {nc} circles (same generator and physics), "
                             f"{len(per)} of {args.steps} requested steps within {args.ref_budget:.0f} s"},
        "cpu_baseline": {"value": value, "unit": "GLUPS", "cores": cores, "kind": "port",
                         "sample": f"oracle/lbm_oracle.c (OpenMP restatement of the reference step incl. its "
                                   f"per-step wall-distance sweep), {cores} threads, {size}x{size}, {len(per)} steps"},
        "e2e": {"value": value, "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


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
    ap.add_argument("--cpu-size", type=int, default=1024)
    ap.add_argument("--ref-budget", type=float, default=150.0, help="seconds cap of the reference arm")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end run (default: --steps)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import lbm2d
    lbm2d.build(quiet=True)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:  # independent replicas, one per GPU: no data-path collective
        import torch.distributed as dist
        dist.init_process_group("gloo")
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
        s.upload_f(f0)
        if dist:
            dist.barrier()
        clocks.active = True
        try:
            ms, kms, launches = time_device(s, torch, args.steps, args.warmup)
            nan = False
        except lbm2d.LBMError as ex:  # a diverged run is reported, not timed
            if ex.code != 4:
                raise
            ms, kms, launches, nan = float("nan"), float("nan"), 0, True
        clocks.active = False
        t = torch.tensor([ms], dtype=torch.float64)
        if dist:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        info = s.info()
        results[label] = dict(ms=float(t[0]), kernel_ms=kms, launches=launches, nan=nan,
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
            if dist:
                dist.barrier()
            clocks.active = True
            e2e_ms, e2e_launches = time_e2e(lbm2d, s, torch, e2e_steps, pin, pout)
            clocks.active = False
            t = torch.tensor([e2e_ms], dtype=torch.float64)
            if dist:
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
            results["e2e"] = dict(ms=float(t[0]), steps=e2e_steps, launches=e2e_launches)
            del pin, pout
        s.close()
    clocks.stop()

    if rank != 0:
        return 0
    nodes = nx * ny
    peak, peak_kind = peaks()
    main_st = storages[0]
    r0 = results[main_st]
    bpu = 2 * 9 * lbm2d.BYTES_PER_POP[main_st]
    value = world * nodes * args.steps / (r0["ms"] * 1e-3) / 1e9
    alg_bytes = nodes * float(bpu)  # populations read once + written once per lattice update
    achieved = alg_bytes / (r0["kernel_ms"] * 1e-3) / 1e9
    tr = traffic_record()
    traffic = None
    if tr and tr.get("storage") == main_st and tr.get("nodes"):
        traffic = float(tr["dram_bytes_per_launch"]) * nodes / float(tr["nodes"])
    prec = {}
    for label, st, les in runs[1:]:
        r = results[label]
        g = world * nodes * args.steps / (r["ms"] * 1e-3) / 1e9
        b = 2 * 9 * lbm2d.BYTES_PER_POP[st]
        kach = nodes * b / (r["kernel_ms"] * 1e-3) / 1e9
        prec[label] = {"glups": g, "vs_" + main_st: g / value, "kernel_ms": r["kernel_ms"], "les": les,
                       "roofline_frac": kach / peak, "bytes_per_update": b, "diverged": r["nan"]}
    e2e = None
    if "e2e" in results:
        e = results["e2e"]
        e2e = {"value": world * nodes * e["steps"] / (e["ms"] * 1e-3) / 1e9, "unit": "GLUPS",
               "h2d_bytes_per_step": nodes * 9 * 8 / e["steps"], "d2h_bytes_per_step": 16 + nodes * 9 * 8 / e["steps"],
               "steps": e["steps"], "launches": e["launches"],
               "note": "initial state H2D from pinned memory + per step (step, drag/lift D2H) + final state D2H"}
    cpu = None
    if not args.no_cpu:
        try:
            cores = os.cpu_count() or 1
            mlups, dt, nc, n = cpu_sample(args.cpu_size)
            cpu = {"value": mlups / 1e3, "unit": "GLUPS", "cores": cores, "kind": "port",
                   "sample": f"oracle/lbm_oracle.c (OpenMP restatement of the reference step, per-step "
                             f"wall-distance sweep included), {cores} threads, same generator and physics at "
                             f"{args.cpu_size}x{args.cpu_size} with {nc} circles, {n} steps in {dt:.1f} s"}
        except Exception as ex:  # the CPU leg never blocks the GPU line
            cpu = {"value": None, "unit": "GLUPS", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {ex}"}
    line = {
        "metric": "GLUPS (D2Q9 step, lattice updates/s) & %HBM roofline, FP32 vs FP16/BF16 storage",
        "value": value, "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r0["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp32": "f32", "fp64": "f64"}.get(main_st, "f32"), "data": "synthetic",
        "config": {"workload": workload_name(nx, ny), "nx": nx, "ny": ny, "storage": main_st, "tau": TAU,
                   "body_force_x": BODY_FORCE, "l2": "inputs larger than L2 (populations >= 129 MB, no flush)",
                   "parallelism": "replicas" if world > 1 else "single GPU", "block": list(r0["block"]),
                   "boundary_nodes": r0["boundary"], "force_nodes": r0["force_nodes"], "diverged": r0["nan"]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                     "kernel_ms": r0["kernel_ms"], "kernel": "step_kernel"},
        "precision": prec,
        "e2e": e2e,
        "gpu_launches": r0["launches"],
        "clocks": clocks.summary(),
        "cpu_baseline": cpu,
        "drag_lift": r0.get("force"),
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
