#!/usr/bin/env python
"""Throughput benchmark of the GB300 level-set solver.

Workload (configuration 3 of the reference's benchmark plan): a 512^3
periodic grid, G0 = perturbed sphere (r0 = 0.2, 8 spherical-harmonic modes),
velocity = curl of a 24-mode random vector potential scaled to max|u| = 1,
S_L = 0.2, dt from CFL 0.5 with the field-max speed, WENO-5 + TVD-RK3, HCR-2
reinitialisation every 5 steps with 2 pseudo-steps.  Fields are seeded
synthetic data generated on the device.

One bench step = one reinitialisation period: 5 TVD-RK3 steps + 1 HCR-2
(2 pseudo-steps).  Metric: Gcell-updates/s = interior cells x RK3 steps /
time.  The headline value is the FP32-bulk form (FP64 interface constraint
and reductions); the plain FP64 form is measured beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's algorithm on the host CPU cores
(the oracle port under oracle/, pinned bit-exact to the reference's own
sources) on the full grid of the same workload, one bench step per step.
Multi-GPU runs are independent replicas (the path is not sharded); rank 0
prints the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "level-set-method-code_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Gcell-updates/s at 512^3 FP32 vs FP64 at stated Linf; adjoint/forward cost ratio"


def l2_note(n: int) -> str:
    """How a stage launch's working set (6 FP32 fields) compares with the 129 MB L2."""
    ws = 6 * n ** 3 * 4
    return (f"inputs larger than L2 (each FP32 field {n ** 3 * 4 / 2 ** 20:.0f} MiB, {ws / 2 ** 20:.0f} MiB per stage)"
            if ws > 129e6 else f"working set {ws / 2 ** 20:.0f} MiB per stage fits in L2 (not flushed)")


def workload_config(n: int, world: int) -> dict:
    """The benchmark's workload, the same for both arms (each states its
    arithmetic in "form")."""
    return {"workload": f"config3 {n}^3 periodic, WENO5-RK3 + HCR-2 (every 5 steps, 2 pseudo-steps), "
                        "S_L=0.2, CFL 0.5",
            "grid": n, "bench_step": "5 RK3 steps + 1 HCR-2 reinit", "parallelism": f"replicas x{world}"}
RK_PER_BENCH_STEP = 5      # reinit interval
REINIT_ITERS = 2
CFL = 0.5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", "--grid", dest="n", type=int, default=512)
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed FP64 bench steps (0 = skip)")
    ap.add_argument("--e2e-steps", type=int, default=2, help="timed end-to-end calls (0 = skip)")
    ap.add_argument("--e2e-rk-steps", type=int, default=50, help="RK3 steps per end-to-end call")
    ap.add_argument("--cpu-seconds", type=float, default=12.0,
                    help="CPU baseline sample length (whole reinit periods on the full grid, at least one)")
    ap.add_argument("--batch-steps", type=int, default=200, help="RK3 steps of the batched form (0 = skip)")
    ap.add_argument("--adjoint-steps", type=int, default=300, help="RK3 steps of the adjoint form (0 = skip)")
    ap.add_argument("--adjoint-n", type=int, default=192)
    ap.add_argument("--sample-steps", type=int, default=10, help="steps of the sample-surface frequency sweep (0 = skip)")
    ap.add_argument("--plane-n", type=int, default=4096, help="grid of the 2D stage-kernel leg (0 = skip)")
    ap.add_argument("--deform-steps", type=int, default=20, help="RK3 steps of the live deformation leg (0 = skip)")
    ap.add_argument("--no-config1", dest="config1", action="store_false", help="skip the 128^2 configuration-1 leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--json-out", default=None)
    ap.add_argument("--clocks-out", default=None, help="write the nvidia-smi clock samples to this CSV file")
    return ap.parse_args()


# -- distributed plumbing (replicas) ------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None

    def init(self, backend):
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = torch.device("cuda", self.local) if torch.cuda.is_available() else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        dev = torch.device("cuda", self.local) if torch.cuda.is_available() else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def done(self):
        if self.pg:
            self.pg.destroy_process_group()


# -- clocks ------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, out_path: str | None = None):
        self.gpu = gpu_index
        self.out_path = out_path
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        self.lines = [l for l in out.splitlines() if l.strip()]
        if self.out_path:
            with open(self.out_path, "w") as f:
                f.write(self.FIELDS + "\n" + "\n".join(self.lines) + "\n")

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [x.strip() for x in l.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# -- helpers -----------------------------------------------------------------
def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(precision: str, n: int):
    """dram bytes per stage-kernel launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "stage_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        d = json.load(f)
    e = d.get(f"{precision}_{n}")
    return None if e is None else float(e["bytes_per_launch"])


def make_solver(lsgb, syn, n: int, precision: str, stream):
    wl = syn.config3(n)
    p = lsgb.params(3, n, n, n, s_l=wl.s_l, enable_reinit=True, reinit_interval=RK_PER_BENCH_STEP,
                    reinit_iterations=REINIT_ITERS)
    s = lsgb.Solver(p, precision)
    s.set_stream(stream)
    s.synth(syn.to_device_desc(wl))
    s.compute_dt(CFL)
    return s, wl


def time_solver(torch, s, stream, steps: int, warmup: int, dist: Dist | None, sampler=None):
    """Returns (elapsed_ms over `steps` bench steps, kernel launches in the window,
    stage_ms, stage_launches, reinit_ms, reinit_launches)."""
    import lsgb
    for _ in range(warmup):
        s.advance(RK_PER_BENCH_STEP)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    s.enable_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = lsgb.launch_count()
    if sampler:
        sampler.start()
        time.sleep(0.3)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(steps):
            s.advance(RK_PER_BENCH_STEP)
        e1.record(stream)
    torch.cuda.synchronize()
    if sampler:
        sampler.stop()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches = lsgb.launch_count() - n0
    ms = e0.elapsed_time(e1)
    st_ms, st_n, re_ms, re_n = s.kernel_times()
    s.enable_timing(False)
    return ms, launches, st_ms, st_n, re_ms, re_n


# -- CPU leg (oracle: the reference's algorithm on the host cores) -------------
def cpu_info() -> dict:
    """Host CPU model (lscpu "Model name") and logical CPU count."""
    import platform
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for l in out.splitlines():
            if l.startswith("Model name:"):
                model = l.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cpu_model": model or platform.processor() or platform.machine(), "host_cpus": os.cpu_count()}


def omp_threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


class CpuRun:
    """The reference's algorithm (the oracle port, oracle/ls_oracle.c, OpenMP
    over all host cores) on the full n^3 grid of the workload: the fields are
    built on the host (lsgb.synthetic.host_fields, FP64, max |u| = 1), dt from
    CFL 0.5 with the field-max speed.  One period = 5 RK3 steps + the HCR-2
    reinitialisation after the 5th (the reference's cadence, steps 1..5)."""

    def __init__(self, n: int):
        from lsgb import synthetic as syn
        from oracle import Oracle, Problem
        self.orc = Oracle("port")
        wl = syn.config3(n)
        self.G, self.u, self.v, self.w = syn.host_fields(wl)
        dt = syn.cfl_dt(wl, self.u, self.v, self.w, CFL)
        self.pb = Problem(nx=n, ny=n, nz=n, dim=3, s_l=wl.s_l, dt=dt, enable_reinit=True,
                          reinit_interval=RK_PER_BENCH_STEP, reinit_iterations=REINIT_ITERS)
        self.cells = n ** 3
        self.periods = 0

    def period(self) -> float:
        """Advances one period; returns its wall time in seconds."""
        a = time.perf_counter()
        self.orc.run_filled(self.pb, RK_PER_BENCH_STEP, self.G, self.u, self.v, self.w,
                            step0=1 + RK_PER_BENCH_STEP * self.periods)
        self.periods += 1
        return time.perf_counter() - a


def cpu_sample(n: int, target_s: float):
    """Bounded CPU sample on the full grid: whole periods until target_s has
    passed (at least one).  Returns (Gcell-updates/s, periods, seconds)."""
    run = CpuRun(n)
    el = 0.0
    while True:
        el += run.period()
        if el >= target_s:
            break
    return run.cells * RK_PER_BENCH_STEP * run.periods / el / 1e9, run.periods, el


def run_reference(args, dist: Dist):
    """--impl reference: the reference algorithm on the host cores, on the
    same full grid and bench steps as the GPU arm."""
    if dist.rank != 0:
        return
    from oracle import build_port
    build_port()
    run = CpuRun(args.n)
    for _ in range(args.warmup):
        run.period()
    timed = [run.period() for _ in range(args.steps)]
    step_s = sum(timed) / len(timed)
    value = run.cells * RK_PER_BENCH_STEP / step_s / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gcell-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded config-3 fields built on the host)",
        "config": {**workload_config(args.n, args.gpus),
                   "form": f"the reference's FP64 arithmetic (oracle port, OpenMP) on the full {args.n}^3 grid"},
        "cpu_baseline": {"value": value, "unit": "Gcell-updates/s", "cores": omp_threads(), "kind": "port",
                         "sample": f"full {args.n}^3 grid, {len(timed)} timed periods of 5 RK3 steps + 1 HCR-2 "
                                   f"after {args.warmup} warm-up periods",
                         **cpu_info()},
        "e2e": {"value": value, "unit": "Gcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def measure_batched(torch, lsgb, syn, steps: int, dist: Dist):
    """Configuration 4: 48 2D (64^2..1024^2) + 48 3D (32^3..192^3) instances,
    FP32-bulk, HCR-2 every 5 steps, tiles from the autotuner, advanced together
    with one captured CUDA graph per reinit period; `steps` RK3 steps timed
    with CUDA events on the batch stream.  The headline is the grouped form
    (one launch per RK3 stage / pseudo-step / copy for all 3D instances and one
    for all 2D ones); the per-instance launches on 16 streams are timed
    beside it ("lanes")."""
    wls = syn.config4()
    out = {}
    for mode in ("grouped", "lanes"):
        cells = 0
        with lsgb.Batch("f32", lanes=16) as b:
            b.set_mode(mode)
            for wl in wls:
                n = wl.n[0]
                p = lsgb.params(wl.dim, n, n, n, s_l=wl.s_l, enable_reinit=True, reinit_interval=RK_PER_BENCH_STEP,
                                reinit_iterations=REINIT_ITERS)
                s = b.add(p)
                s.synth(syn.to_device_desc(wl))
                s.compute_dt(CFL)
                cells += n ** wl.dim
            t0 = time.perf_counter()
            b.autotune()
            tune_s = time.perf_counter() - t0
            tiles = [s.get_tile() for s in b.instances]
            b.advance(6)  # warm-up: direct step 0 + the captured period
            b.sync()
            stream = torch.cuda.ExternalStream(b.stream_handle())
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n0 = lsgb.launch_count()
            e0.record(stream)
            b.advance(steps)
            e1.record(stream)
            b.sync()
            ms = e0.elapsed_time(e1)
            launches = lsgb.launch_count() - n0
            replays, kernels = b.stats()
            used = b.mode
        ms = dist.max(ms)
        out[mode] = {"value": dist.world * cells * steps / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s",
                     "mode": used, "instances": len(wls), "cells_per_step": cells, "rk3_steps": steps, "ms": ms,
                     "kernels_launched": launches, "graph_replays": replays, "kernels_per_graph": kernels,
                     "autotune_s": tune_s, "tiles_2d": sorted(set(t for t, w in zip(tiles, wls) if w.dim == 2)),
                     "tiles_3d": sorted(set(t for t, w in zip(tiles, wls) if w.dim == 3))}
    res = dict(out["grouped"])
    res["lanes"] = {k: out["lanes"][k] for k in ("value", "ms", "kernels_per_graph", "kernels_launched", "tiles_3d")}
    res["workload"] = "config4: 48 2D (64^2..1024^2) + 48 3D (32^3..192^3), FP32-bulk, reinit every 5"
    return res


def measure_plane(torch, lsgb, syn, n: int, steps: int, peak_gbs: float, dist: Dist):
    """The 2D FP32 stage kernel on one n x n plane (periodic): the first 2D
    instance of configuration 4 (circle, 8-mode divergence-free velocity,
    its S_L) at n^2, HCR-2 every 5 steps.  Stage launches of `steps` RK3
    steps timed with the handle's CUDA events; algorithmic bytes per launch:
    G, u, v in and G' out (16 B per cell), plus G^n in stages 2 and 3."""
    wl = syn.config4(1, 0)[0]
    wl.n = (n, n)
    p = lsgb.params(2, n, n, 1, s_l=wl.s_l, enable_reinit=True, reinit_interval=RK_PER_BENCH_STEP,
                    reinit_iterations=REINIT_ITERS)
    with lsgb.Solver(p, "f32") as s:
        s.synth(syn.to_device_desc(wl))
        s.compute_dt(CFL)
        s.advance(RK_PER_BENCH_STEP)  # warm-up, one reinit period
        s.enable_timing(True)
        s.advance(steps)
        st, sn, rt, rn = s.kernel_times()
        s.enable_timing(False)
    st, rt = dist.max(st), dist.max(rt)
    ms = st / max(sn, 1)
    alg = n * n * 4 * (4 + 5 + 5) / 3  # average over the three stages
    return {"stage_avg_launch_ms": ms, "stage_launches": sn, "reinit_avg_launch_ms": rt / max(rn, 1),
            "gcell_stage_per_s": n * n / (ms * 1e-3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": peak_gbs, "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / peak_gbs, "algorithmic_bytes_per_launch": alg},
            "kernel": "stage2d_f32_rows (fused WENO5 RHS + RK3 stage combine, 32 x 32 row-pair tiles)",
            "workload": f"{n}^2 periodic plane, config-4 2D instance 0 construction, FP32-bulk, reinit every 5"}


def measure_config1(torch, lsgb, syn, dist: Dist, cpu: bool):
    """Configuration 1, the reference's CPU-runnable case: 2D 128^2 periodic,
    circle r = 0.25, u = (1, 0), S_L = 0.1, dt = 0.5 dx / 1.1, 400 RK3 steps,
    HCR-2 every 10 steps x 5 pseudo-steps, plain FP64 (bit-exact to the
    reference's run: tests/test_gpu_parity.py::test_golden_config1).  The
    fields stay resident; the 400 steps are timed with CUDA events on the
    solver's stream.  The CPU figure is the oracle port of the same run."""
    n, steps = 128, 400
    G, u, v, _ = syn.host_fields(syn.config1(n))
    dt = 0.5 * (1.0 / n) / 1.1
    p = lsgb.params(2, n, n, 1, s_l=0.1, dt=dt, enable_reinit=True, reinit_interval=10, reinit_iterations=5)
    stream = torch.cuda.Stream()
    times = []
    for _ in range(2):  # the first run warms up
        with lsgb.Solver(p, "f64") as s:
            s.set_stream(stream)
            s.set_fields(G, u, v)
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            with torch.cuda.stream(stream):
                ev[0].record(stream)
                s.advance(steps)
                ev[1].record(stream)
            torch.cuda.synchronize()
            times.append(ev[0].elapsed_time(ev[1]))
    ms = dist.max(times[-1])
    out = {"value": dist.world * n * n * steps / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s", "ms": ms,
           "rk3_steps": steps, "dtype": "f64",
           "workload": "config1 128^2 periodic circle, u = (1, 0), S_L = 0.1, CFL 0.5, HCR-2 every 10 x 5"}
    if cpu:
        from oracle import Oracle, Problem
        pb = Problem(nx=n, ny=n, dim=2, s_l=0.1, dt=dt, enable_reinit=True, reinit_interval=10,
                     reinit_iterations=5, periodic_y=True)
        a = time.perf_counter()
        Oracle("port").run(pb, steps, G, u, v)
        el = time.perf_counter() - a
        out["cpu_baseline"] = {"value": n * n * steps / el / 1e9, "unit": "Gcell-updates/s",
                               "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1)),
                               "kind": "port", "sample": f"the whole run, {el:.2f} s"}
    return out


def measure_deformation(torch, lsgb, syn, n: int, steps: int, dist: Dist):
    """The reference's time-dependent case at n^3, FP32: the deformation
    vortex recomputed every step (Local_code/level-set_MPI_3D/src/main.cpp:
    291-317), HCR-2 every 5 steps, on the configuration-3 front.  Two forms of
    the same loop, CUDA events on the solver's stream: the vortex evaluated
    inside the stage kernel (live mode, one advance call) and the explicit
    per-step refill of the stored u, v, w (set_velocity_deformation +
    advance(1)); the two forms give the same bits
    (tests/test_gpu_live_velocity.py)."""
    stream = torch.cuda.Stream()
    s, wl = make_solver(lsgb, syn, n, "f32", stream)
    dt = 0.5 / (n * (2.0 + 1.0 + 1.0 + wl.s_l))  # CFL 0.5: max |u| + |v| + |w| of the vortex is 4
    s.set_dt(dt)
    out = {}
    for form in ("fused", "refill"):
        s.step = 0
        t = 0.0
        if form == "fused":
            s.set_velocity_deformation_live(t, 1.5)
            s.advance(RK_PER_BENCH_STEP)  # warm-up
        else:
            for _ in range(RK_PER_BENCH_STEP):
                s.set_velocity_deformation(t, 1.5)
                s.advance(1)
                t += dt
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            if form == "fused":
                s.advance(steps)
            else:
                for _ in range(steps):
                    s.set_velocity_deformation(t, 1.5)
                    s.advance(1)
                    t += dt
            ev[1].record(stream)
        torch.cuda.synchronize()
        ms = dist.max(ev[0].elapsed_time(ev[1]))
        out[form] = {"ms_per_step": ms / steps, "value": dist.world * n ** 3 * steps / (ms * 1e-3) / 1e9}
    s.close()
    return {"value": out["fused"]["value"], "unit": "Gcell-updates/s", "rk3_steps": steps,
            "ms_per_step": out["fused"]["ms_per_step"], "refill_per_step": out["refill"],
            "workload": f"{n}^3 deformation vortex recomputed every step, FP32, HCR-2 every 5, dt {dt:.3g}"}


def measure_adjoint(torch, lsgb, n: int, steps: int, dist: Dist):
    """Configuration 5: gradient of the smoothed-Heaviside front mismatch with
    respect to the per-cell flame speed S_L(x) at n^3 (FP32-bulk), through
    the discrete adjoint with checkpoints every 20 steps.  Times one plain
    forward of `steps` RK3 steps and the forward-with-checkpoints + loss +
    backward, both with CUDA events on the solver's stream."""
    import numpy as np
    from lsgb import adjoint as adj
    p, G0, u, v, w, sl, sl_t = adj.workload(n, steps)
    stream = torch.cuda.Stream()
    prob = adj.Problem(p, G0, u, v, w, "f32", checkpoint=20)
    prob.a.set_grads(sl=True, velocity=False)  # the workload's gradient is dL/dS_L
    prob.s.set_stream(stream)
    prob.target(sl_t, steps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    prob.run(sl, steps)  # warm
    prob.s.volume()
    prob.run(sl, 0)
    ev[0].record(stream)
    prob.s.advance(steps)
    ev[1].record(stream)
    prob.s.volume()
    prob.run(sl, 0)
    n0 = lsgb.launch_count()
    ev[2].record(stream)
    prob.a.forward(steps)
    loss = prob.a.loss(seed=True)
    prob.a.backward()
    ev[3].record(stream)
    torch.cuda.synchronize()
    launches = lsgb.launch_count() - n0
    fwd_ms = dist.max(ev[0].elapsed_time(ev[1]))
    adj_ms = dist.max(ev[2].elapsed_time(ev[3]))
    g = prob.a.grad("sl")
    prob.close()
    cells = n ** 3
    return {"value": dist.world * cells * steps / (adj_ms * 1e-3) / 1e9, "unit": "Gcell-updates/s (forward+backward)",
            "forward_ms": fwd_ms, "forward_backward_ms": adj_ms, "adjoint_over_forward": adj_ms / fwd_ms,
            "loss": loss, "grad_l2": float(np.linalg.norm(g)), "kernels_launched": launches,
            "rk3_steps": steps, "checkpoint_interval": 20,
            "workload": f"config5 {n}^3 periodic, FP32-bulk, S_L(x) = 0.15 + 0.05 f(x) (8 modes), "
                        "reinit every 10, L = 1/2 sum (H(G_T) - H(G_target))^2 dV, eps = 1.5 dx"}


def measure_sample(torch, lsgb, steps: int, dist: Dist, cpu: bool):
    """The reference's sample surface as its frequency sweep runs it: 30
    Bunsen-flame instances of 800 x 800 (forcing 5..50 step 5, 55..100 step 5,
    110..200 step 10 Hz; sample/submit_all.sh), LLF WENO-5 + RK3 with the
    anchored/periodic boundaries, FP64 and bit-exact.  One lsgb_sample_run
    call advances all instances `steps` steps (CUDA events on its stream).
    The CPU figure is the oracle port of the same loop on one instance."""
    from lsgb import sample as smp
    freqs = list(range(5, 51, 5)) + list(range(55, 101, 5)) + list(range(110, 201, 10))
    nx, ny = smp.NX, smp.NY
    dx, dy = smp.spacing(nx, ny)
    G0 = torch.tensor(smp.bunsen(nx, ny), dtype=torch.float64, device="cuda")
    stack = G0.unsqueeze(0).repeat(len(freqs), 1, 1).contiguous()
    stream = torch.cuda.Stream()
    t = smp.run(stack, G0, 2, dx, dy, freqs, stream=stream)  # warm
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ev[0].record(stream)
    smp.run(stack, G0, steps, dx, dy, freqs, t=t, stream=stream)
    ev[1].record(stream)
    torch.cuda.synchronize()
    ms = dist.max(ev[0].elapsed_time(ev[1]))
    cells = len(freqs) * nx * ny
    out = {"value": dist.world * cells * steps / (ms * 1e-3) / 1e9, "unit": "Gcell-updates/s", "instances": len(freqs),
           "grid": [nx, ny], "steps": steps, "ms": ms, "dtype": "f64",
           "workload": "sample/main.cpp Bunsen flame, 30 forcing frequencies 5-200 Hz, 800x800, DT 2.5e-6, S_L 0.4"}
    if cpu:
        from oracle import SampleOracle
        so = SampleOracle("port")
        g0 = smp.bunsen(nx, ny)
        g, tc, n_cpu = g0, 0.0, 0
        a = time.perf_counter()
        while time.perf_counter() - a < 8.0:  # about 8 s of host work, whole chunks of 20 steps
            g, tc = so.run(g, g0, 20, dx, dy, smp.DT, smp.SL, smp.U0, smp.V0, smp.EPS_U, smp.EPS_V, 5, tc)
            n_cpu += 20
        el = time.perf_counter() - a
        out["cpu_baseline"] = {"value": nx * ny * n_cpu / el / 1e9, "unit": "Gcell-updates/s",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": f"one instance, {n_cpu} steps, {el:.2f} s"}
    return out


def run_ours(args, dist: Dist):
    import numpy as np
    import torch
    import __graft_entry__ as ge

    ge.build_library()
    import lsgb
    from lsgb import synthetic as syn

    torch.cuda.set_device(dist.local)
    dist.init("nccl")
    n = args.n
    cells = n ** 3
    stream = torch.cuda.Stream()
    clocks_out = None
    if args.clocks_out:
        root, ext = os.path.splitext(args.clocks_out)
        clocks_out = args.clocks_out if dist.world == 1 else f"{root}_rank{dist.rank}{ext}"
    sampler = ClockSampler(dist.local, clocks_out)

    # --- FP32-bulk headline ---
    s32, wl = make_solver(lsgb, syn, n, "f32", stream)
    dt = s32.params().dt
    ms, launches, st_ms, st_n, re_ms, re_n = time_solver(torch, s32, stream, args.steps, args.warmup, dist, sampler)
    ms_max = dist.max(ms)
    rk_steps = args.steps * RK_PER_BENCH_STEP
    value = dist.world * cells * rk_steps / (ms_max * 1e-3) / 1e9

    # roofline of the dominant kernel (the fused RK3 stage): stage 1 moves
    # G, u, v, w in and G1 out (5 fields), stages 2 and 3 also read G^n (6)
    s_bytes = 4
    stage_bytes_total = cells * s_bytes * 17 * rk_steps
    peak, peak_kind = load_peaks()
    achieved = stage_bytes_total / (st_ms * 1e-3) / 1e9
    traffic = load_traffic("f32", n)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                "kernel": "stage3d_f32_col2 (fused WENO5 RHS + RK3 stage combine, TMA-fed 2.5D tiles, register-blocked in y and z)",
                "algorithmic_bytes_per_launch": cells * s_bytes * 17 / 3,
                "launches": st_n, "avg_launch_ms": st_ms / max(st_n, 1)}
    step_bytes = cells * s_bytes * (17 + (4 + 5 * REINIT_ITERS) / RK_PER_BENCH_STEP)
    whole_step_gbs = step_bytes * rk_steps / (ms * 1e-3) / 1e9
    clocks = sampler.summary()

    # --- end to end through the public C ABI with host buffers ---
    e2e = None
    if args.e2e_steps > 0:
        shape = (n + 6,) * 3
        host = [torch.empty(shape, dtype=torch.float64, pin_memory=True) for _ in range(5)]
        for name, t in zip(("G", "u", "v", "w"), host[:4]):
            s32.get_field(name, out=t.numpy())
        s32.run_host(host[0].numpy(), host[1].numpy(), host[2].numpy(), host[3].numpy(), args.e2e_rk_steps,
                     host[4].numpy())  # warm
        # the host link's rate right now (one field each way, median of three
        # copies): it varies by box and sets the end-to-end figure's copy time
        link = {}
        probe = torch.empty(shape, dtype=torch.float64, device="cuda")

        def copy_rate(dst, src):
            e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            e[0].record(stream)
            dst.copy_(src, non_blocking=True)
            e[1].record(stream)
            e[1].synchronize()
            return probe.numel() * 8 / (e[0].elapsed_time(e[1]) * 1e-3) / 1e9

        with torch.cuda.stream(stream):
            for name, dst, src in (("h2d_gbs", probe, host[0]), ("d2h_gbs", host[4], probe)):
                rates = [copy_rate(dst, src) for _ in range(3)]
                link[name] = statistics.median(rates)
                link[name + "_samples"] = rates
            # every input array once (separate pinned allocations: G, u, v, w)
            link["h2d_gbs_per_array"] = [copy_rate(probe, src) for src in host[:4]]
        del probe
        torch.cuda.synchronize()
        dist.barrier()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.e2e_steps + 1)]
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for q in range(args.e2e_steps):
                s32.run_host(host[0].numpy(), host[1].numpy(), host[2].numpy(), host[3].numpy(),
                             args.e2e_rk_steps, host[4].numpy())
                ev[q + 1].record(stream)
        torch.cuda.synchronize()
        e2e_ms = dist.max(ev[0].elapsed_time(ev[-1]))
        per_call = [ev[q].elapsed_time(ev[q + 1]) for q in range(args.e2e_steps)]
        e2e = {"value": dist.world * cells * args.e2e_rk_steps * args.e2e_steps / (e2e_ms * 1e-3) / 1e9,
               "unit": "Gcell-updates/s", "h2d_bytes_per_step": 4 * shape[0] ** 3 * 8,
               "d2h_bytes_per_step": shape[0] ** 3 * 8,
               "call": "lsgb_solver_run_host (ghosted FP64 host arrays G,u,v,w in, G out)",
               "rk3_steps_per_call": args.e2e_rk_steps, "ms_per_call": per_call, "host_link": link}
        del host

    # --- plain FP64 form beside it, and the FP32-vs-FP64 error after the same steps ---
    fp64 = None
    prec = None
    if args.fp64_steps > 0:
        s64, _ = make_solver(lsgb, syn, n, "f64", stream)
        s64.set_dt(dt)
        ms64, _, st64, stn64, _, _ = time_solver(torch, s64, stream, args.fp64_steps, 1, None)
        v64 = dist.world * cells * args.fp64_steps * RK_PER_BENCH_STEP / (dist.max(ms64) * 1e-3) / 1e9
        fp64 = {"value": v64, "unit": "Gcell-updates/s", "ms_per_step": ms64 / args.fp64_steps,
                "stage_avg_launch_ms": st64 / max(stn64, 1),
                "fp32_speedup": value / v64}
        total_periods = 1 + args.fp64_steps
        # FP32 from the same initial state for the same number of steps
        s32b, _ = make_solver(lsgb, syn, n, "f32", stream)
        s32b.set_dt(dt)
        s32b.advance(total_periods * RK_PER_BENCH_STEP)
        g64 = s64.get_G(layout="compact")
        g32 = s32b.get_G(layout="compact")
        d = np.abs(g32 - g64)
        band = np.abs(g64) < 3.0 / n
        prec = {"rk3_steps": total_periods * RK_PER_BENCH_STEP,
                "linf_G": float(d.max()), "linf_G_band3": float(d[band].max()) if band.any() else None,
                "linf_G_band3_over_dx": (float(d[band].max()) * n) if band.any() else None,
                "volume_f64": s64.volume()[0], "volume_f32": s32b.volume()[0]}
        s64.close()
        s32b.close()
        del g64, g32, d, band

    s32.close()

    # --- batched form: 96 uneven 2D/3D instances, one CUDA graph per reinit period ---
    batched = None
    if args.batch_steps > 0:
        batched = measure_batched(torch, lsgb, syn, args.batch_steps, dist)

    config1 = None
    if args.config1:
        config1 = measure_config1(torch, lsgb, syn, dist, cpu=not args.no_cpu_baseline and dist.rank == 0
                                  and dist.world == 1)

    deform = None
    if args.deform_steps > 0:
        deform = measure_deformation(torch, lsgb, syn, n, args.deform_steps, dist)

    plane = None
    if args.plane_n > 0:
        plane = measure_plane(torch, lsgb, syn, args.plane_n, 20, roofline["peak"], dist)

    sample = None
    if args.sample_steps > 0:
        sample = measure_sample(torch, lsgb, args.sample_steps, dist,
                                cpu=not args.no_cpu_baseline and dist.rank == 0 and dist.world == 1)

    adjoint = None
    if args.adjoint_steps > 0:
        adjoint = measure_adjoint(torch, lsgb, args.adjoint_n, args.adjoint_steps, dist)

    cpu = None
    if not args.no_cpu_baseline and dist.rank == 0 and dist.world == 1:
        rate, periods, el = cpu_sample(n, args.cpu_seconds)
        cpu = {"value": rate, "unit": "Gcell-updates/s", "cores": omp_threads(), "kind": "port",
               "sample": f"full {n}^3 grid of the workload, {periods} reinit periods "
                         f"({periods * RK_PER_BENCH_STEP} RK3 steps), {el:.1f} s", **cpu_info()}

    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Gcell-updates/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded config-3 fields generated on the device)",
            "config": {**workload_config(n, dist.world),
                       "form": "FP32-bulk WENO5-RK3 + HCR-2, FP64 interface constraint and reductions", "dt": dt,
                       "l2": l2_note(n)},
            "roofline": roofline,
            "whole_step_algorithmic_GBps": whole_step_gbs,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
            "fp64": fp64,
            "precision_vs_fp64": prec,
            "reinit_avg_launch_ms": re_ms / max(re_n, 1),
            "config1": config1,
            "plane2d": plane,
            "deformation": deform,
            "batched": batched,
            "adjoint": adjoint,
            "sample_sweep": sample,
        }
        s = json.dumps(line)
        print(s, flush=True)
        if args.json_out:
            with open(args.json_out, "w") as f:
                f.write(s + "\n")
    dist.done()


def main():
    args = parse()
    dist = Dist()
    if args.impl == "reference":
        run_reference(args, dist)
        return
    run_ours(args, dist)


if __name__ == "__main__":
    main()
