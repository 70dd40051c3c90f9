#!/usr/bin/env python
"""Throughput benchmark of the FDTD time-stepping hot path.

Workload: the dispersive-scattering configuration (ffip_gb300.workloads.
dispersive_spheres(256)): 256^3 Yee cells, 16-cell CPML, 64 Lorentz/Drude
spheres, an Ex current sheet, a 128x128x32 Ex DFT monitor at 5 frequencies.
One "step" is one FDTD time step (H and E half steps with CPML, ADE and DFT)
over the whole grid.  Metric: Yee cell-updates per second (256^3 per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm (default) times K steps of the fp32-state stepper (fp64 DFT sums) with
CUDA events on the stepper's stream, inputs resident in HBM; the state (about
0.9 GB) is far larger than the 129 MB L2, so no flush is needed between steps.
It also reports the fp64 stepper, the fp32-vs-fp64 DFT error of a full
4000-step run, an end-to-end figure through the C ABI (config in, DFT arrays
out, set-up and copies inside the timed region), the roofline of the step
kernel(s) and a CPU baseline (the oracle's restatement of the reference's
loops on all host cores, a bounded sample of steps).

--impl reference times that CPU restatement of the reference's own loops
(oracle/port.py + oracle/step.c) on the host cores, K steps after W warm-up
steps, on the same workload.

Multi-GPU: the stepper does not shard here (one GPU per box); with torchrun
each rank runs an independent replica on its own GPU ("replicas only"),
value = all ranks' cell-updates / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Yee cell-updates/s (fp32 state, fp64 DFT), dispersive 256^3"
UNIT = "Gcell-updates/s"


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(v)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return v


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms; start() /
    stop() bracket the timed region, and summary() keeps the samples whose
    nvidia-smi timestamp falls inside it."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.p = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def start(self):
        self.t0 = datetime.datetime.now()

    def stop(self):
        self.t1 = datetime.datetime.now()

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.t.join(timeout=5)

    @staticmethod
    def _when(r):
        try:
            return datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f")
        except (ValueError, IndexError):
            return None

    def summary(self, timed=None):
        """Samples inside [start, stop]: the whole fp32 leg (warm-up, the K
        timed steps and the full-length fp32 run, all the same kernels at the
        same load), so that a short timed region (20 steps last about 9 ms,
        shorter than the 50 ms sampling period) still has a clock record;
        timed: (t0, t1) of the K timed steps, whose own samples are counted
        apart."""
        rows = [r for r in self.rows if len(r) >= 10]
        inside = rows
        if self.t0 is not None and self.t1 is not None:
            inside = [r for r in rows if (w := self._when(r)) is not None and self.t0 <= w <= self.t1]
        n_timed = None
        if timed is not None:
            n_timed = sum(1 for r in rows if (w := self._when(r)) is not None and timed[0] <= w <= timed[1])
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0, "samples_total": len(rows),
                    "samples_timed_steps": n_timed}
        num = lambda v: float(v) if v.replace(".", "").isdigit() else None  # noqa: E731
        sm = [x for x in (num(r[2]) for r in inside) if x is not None]
        mx = [x for x in (num(r[3]) for r in inside) if x is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in inside:
            for i, n in enumerate(names):
                if r[6 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(inside), "samples_total": len(rows),
                "samples_timed_steps": n_timed,
                "window_s": (self.t1 - self.t0).total_seconds() if self.t0 else None,
                "sampling": "nvidia-smi every 50 ms; samples timestamped inside the fp32 leg (warm-up, the timed "
                            "steps and the full-length fp32 run)"}


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(n):
    """DRAM bytes per k_fused launch from the committed ncu summary of the
    n^3 workload (dram__bytes_read.sum + dram__bytes_write.sum), or None."""
    p = os.path.join(ROOT, "profiles", "k_fused_fp32_dispersive%d.md" % n)
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.startswith("| DRAM traffic per launch |"):
                return float(line.split("|")[2].split()[0]) * 1e6
    return None


def dft_rel_err(a, b):
    g = "volume fields dft 0"
    scale = max(np.abs(b[g]["real"]).max(), np.abs(b[g]["imag"]).max())
    return float(max(np.abs(a[g]["real"] - b[g]["real"]).max(), np.abs(a[g]["imag"] - b[g]["imag"]).max()) / scale)


def cpu_leg(cfg, steps, warmup, threads):
    """The oracle's restatement of the reference's stepping loops, timed."""
    from oracle import port
    t0 = time.perf_counter()
    sim = port.OracleSim(cfg, {}, threads=threads)
    setup = time.perf_counter() - t0
    sim.run_steps(warmup)
    t0 = time.perf_counter()
    sim.run_steps(steps)
    dt = time.perf_counter() - t0
    return dt, setup


def large_leg(dev, steps=100):
    """The large design workload's forward simulation (workloads.large_design:
    512 x 512 x 384 cells, 24-cell CPML, Drude backplane, 256 x 256 x 32
    Lorentz/vacuum design box, three 256 x 256 DFT planes at 16 frequencies),
    fp32 state: set-up time and device-timed step rate.  One design
    iteration there is a forward run and one adjoint run per objective
    frequency, 20000 steps each."""
    from ffip_gb300 import native, workloads
    cfg, ds = workloads.large_design(precision="fp32")
    cfg["device"] = dev
    t0 = time.perf_counter()
    s = native.NativeSim(cfg, ds)
    setup = time.perf_counter() - t0
    s.step(3)
    s.sync()
    ms, pms = s.step_timed_pass(steps)
    ms, pms = ms / steps, pms / steps
    st = s.stats()
    s.close()
    cells = st["yee_cells"]
    run_s = 20000 * ms / 1e3
    return {"workload": "large design 512x512x384, 24-cell CPML, Drude backplane, 256x256x32 Lorentz/vacuum design box, "
                        "3 DFT planes x 16 freqs, fp32 state", "cells": cells, "steps_timed": steps, "ms_per_step": ms,
            "gcell_updates_per_s": cells / ms / 1e6, "achieved_gbs": st["bytes_per_step"] / (ms * 1e-3) / 1e9,
            "pass_ms": pms, "pass_achieved_gbs": st["bytes_per_step"] / (pms * 1e-3) / 1e9 if pms > 0 else None,
            "setup_s": setup, "seconds_per_20000_step_run": run_s,
            "seconds_per_design_iter_1fwd_16adj": 17 * run_s}


def set_density_leg(dev):
    """One design iteration's media update (ffip_set_density: new density,
    media re-derived, fields reset) on the adjoint workload's forward
    simulation (192 x 192 x 160 cells, 96 x 96 x 24 two-medium box, 97 x 97
    x 25 density nodes) and on the large design grid (512 x 512 x 384 cells,
    256 x 256 x 32 Lorentz/vacuum box, 257 x 257 x 33 nodes): median wall
    time of 3 updates with the media rasterised on the GPU and on the host."""
    from ffip_gb300 import native, workloads
    prob, rho = workloads.adjoint_design(precision="fp32")
    cfg = prob.forward_simulation.config(prob.stop)
    ds = prob.forward_simulation.dump()
    name = [k for k in ds if k.startswith("two medium box")][0]
    big_cfg, big_ds = workloads.large_design(precision="fp32")
    out = {}
    for label, (c0, d0, nm, r0) in (("adjoint_design_192x192x160", (cfg, ds, name, rho)),
                                    ("large_design_512x512x384", (big_cfg, big_ds, "two medium box 0",
                                                                  big_ds["two medium box 0"]))):
        res = {}
        for mode in ("device", "host"):
            c = dict(c0)
            c["rasterize"] = mode
            c["device"] = dev
            s = native.NativeSim(c, d0)
            times = []
            rng = np.random.default_rng(5)
            for _ in range(3):
                r2 = np.clip(np.asarray(r0) + 0.05 * rng.normal(size=np.shape(r0)), 0, 1)
                s.sync()
                t0 = time.perf_counter()
                s.set_density(nm, r2)
                s.sync()
                times.append(time.perf_counter() - t0)
            s.close()
            res[mode + "_ms"] = statistics.median(times) * 1e3
        out[label] = res
    return out


def vacuum64_leg(dev, cpu):
    """The plain fp64 vacuum box (64^3, 8-cell CPML, one Ez point current,
    Ez DFT plane at 3 frequencies, 1000 steps): GPU fp64 device time, and the
    oracle's restatement of the reference's loops on the host cores."""
    from ffip_gb300 import native, workloads
    cfg = workloads.vacuum_point(64, steps=1000, precision="fp64")
    cfg["device"] = dev
    s = native.NativeSim(cfg)
    s.step(10)
    ms = s.step_timed(1000)
    cells = s.stats()["yee_cells"]
    s.close()
    out = {"workload": "vacuum 64^3, 8-cell CPML, Ez point source, 1000 steps, fp64", "gpu_ms_per_step": ms / 1000,
           "gpu_gcell_updates_per_s": cells * 1000 / (ms * 1e-3) / 1e9}
    if cpu:
        threads = os.cpu_count() or 1
        dt, _ = cpu_leg(workloads.vacuum_point(64, steps=1000, precision="fp64"), 200, 5, threads)
        out["cpu_gcell_updates_per_s"] = cells * 200 / dt / 1e9
        out["cpu_cores"] = threads
        out["cpu_sample"] = "200 steps after 5 warm-up steps"
        out["gpu_over_cpu"] = out["gpu_gcell_updates_per_s"] / out["cpu_gcell_updates_per_s"]
    return out


def design_leg(iters, dev, world):
    """Seconds per design iteration on the adjoint workload: 192 x 192 x 160
    cells, 16-cell CPML, 96 x 96 x 24 design box (97 x 97 x 25 density nodes,
    seeded filtered noise, eps = 1 + 11 rho), Ex sheet below, |Ex|^2 at 4
    probe cells above at 3 frequencies; fp32 state; one forward run and one
    broadband adjoint run (all three frequencies) of 5000 steps per
    iteration, then the gradient on the density nodes.  The first iteration
    (which also builds the two device simulations) is reported apart; each
    timed iteration takes a small gradient step, so densities and adjoint
    sources change every time; its forward part (density update, run,
    objective) and adjoint part (adjoint sources, run, sensitivity) are timed
    apart too."""
    from ffip_gb300 import workloads
    prob, rho = workloads.adjoint_design(precision="fp32")
    for sim in [prob.forward_simulation] + [t.adjoint_simulation for t in prob.terms]:
        sim.device = dev
    barrier(world)
    t0 = time.perf_counter()
    F, g = prob.value_and_gradient(rho)
    first = time.perf_counter() - t0
    times, values, fwd_s, adj_s = [], [F], [], []
    for _ in range(iters):
        step = 0.002 / max(np.abs(g).max(), 1e-30)
        rho = np.clip(rho - step * g, 0.0, 1.0)
        barrier(world)
        t0 = time.perf_counter()
        F = prob.forward(rho)
        t1 = time.perf_counter()
        g = prob.gradient()
        t2 = time.perf_counter()
        times.append(allmax(world, t2 - t0))
        fwd_s.append(t1 - t0)
        adj_s.append(t2 - t1)
        values.append(F)
    prob.release()
    steps = int(round(prob.stop.time / 0.5))
    cells = 192 * 192 * 160
    return {"value": statistics.median(times), "unit": "s/design iter", "first_iter_s": first,
            "iters_timed": iters, "runs_per_iter": 1 + len(prob.terms), "steps_per_run": steps,
            "forward_s": statistics.median(fwd_s), "adjoint_and_gradient_s": statistics.median(adj_s),
            "gcell_updates_per_s": (1 + len(prob.terms)) * steps * cells / statistics.median(times) / 1e9,
            "objective": values, "dtype": "f32 state, f64 DFT and gradient",
            "workload": "adjoint design 192x192x160, 16-cell CPML, 96x96x24 design box, Ex sheet, "
                        "|Ex|^2 at 4 probes x 3 freqs, 5000 steps per run"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--cells", dest="n", type=int, default=256, help="cells per axis of the workload")
    ap.add_argument("--cpu-steps", type=int, default=8, help="steps timed for the CPU baseline sample")
    ap.add_argument("--skip-full-run", action="store_true", help="skip the full-length fp32/fp64 runs")
    ap.add_argument("--engine", default="auto")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--fp32-only", action="store_true", help="time only the fp32 stepper (profiling runs)")
    ap.add_argument("--no-large", action="store_true", help="skip the large design workload's step rate")
    ap.add_argument("--design-iters", type=int, default=2,
                    help="timed design iterations of the adjoint workload (0: skip that leg)")
    a = ap.parse_args()
    world, rank, local = dist_init()
    from ffip_gb300 import workloads
    warm = max(3, a.warmup)
    n = a.n
    cells = float(n) ** 3
    cfg_meta = {"workload": "dispersive spheres %d^3, 16-cell CPML, 64 Lorentz/Drude spheres, Ex sheet, "
                            "128x128x32 Ex DFT x5 freqs" % n if n == 256 else "dispersive spheres %d^3" % n,
                "cells": int(cells), "steps_full_run": workloads.dispersive_spheres(n)["stop condition"]["time"] / 0.5,
                "l2": "state (~0.9 GB fp32) exceeds the 129 MB L2; no flush needed",
                "parallelism": "replicas" if world > 1 else "single GPU"}

    if a.impl == "reference":
        if rank != 0:
            return 0
        threads = os.cpu_count() or 1
        cfg = workloads.dispersive_spheres(n, precision="fp64")
        dt, setup = cpu_leg(cfg, a.steps, warm, threads)
        v = cells * a.steps / dt / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
                "warmup": warm, "ms_per_step": dt / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg_meta,
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "cpu_model": cpu_model(), "kind": "port",
                                 "sample": "%d time steps of the full workload after %d warm-up steps (set-up %.1f s untimed)"
                                           % (a.steps, warm, setup)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    from ffip_gb300 import native
    native.load()
    dev = local
    peak, peak_kind = peaks()

    def make(prec):
        cfg = workloads.dispersive_spheres(n, precision=prec, engine=a.engine)
        cfg["device"] = dev
        return cfg

    def full_run(prec):
        """One full-length run through the C ABI: config in, set-up, stepping,
        DFT arrays out (wall clock, max over ranks)."""
        barrier(world)
        t0 = time.perf_counter()
        s = native.NativeSim(make(prec))
        s.run()
        o = s.outputs()
        dt = time.perf_counter() - t0
        st = s.stats()
        s.close()
        return o, allmax(world, dt), st

    # ---- device-resident throughput, fp32 and fp64
    res = {}
    clocks = None
    full = {}
    e2e = None
    for prec in (("fp32",) if a.fp32_only else ("fp32", "fp64")):
        s = native.NativeSim(make(prec))
        # the clock sampler runs over the whole fp32 leg: from before the
        # warm-up (nvidia-smi takes a moment to start) through the timed
        # steps and the full-length fp32 run
        cs = ClockSampler(dev).__enter__() if prec == "fp32" else None
        if cs:
            time.sleep(0.3)
            cs.start()
        s.step(warm)
        s.sync()
        st0 = s.stats()
        barrier(world)
        ta = datetime.datetime.now()
        ms, pass_ms = s.step_timed_pass(a.steps)
        tb = datetime.datetime.now()
        barrier(world)
        st1 = s.stats()
        ms = allmax(world, ms)
        pass_ms = allmax(world, pass_ms)
        res[prec] = {"ms": ms, "pass_ms": pass_ms, "launches": st1["kernel_launches"] - st0["kernel_launches"],
                     "bytes_per_step": st1["bytes_per_step"], "pass_bytes_per_step": st1["pass_bytes_per_step"],
                     "fused": st1["fused"]}
        s.close()
        if prec == "fp32" and not a.skip_full_run:
            o, dt, st = full_run("fp32")
            full["fp32"] = o
            steps_run = st["time_step"]
            e2e = {"value": world * cells * steps_run / dt / 1e9, "unit": UNIT,
                   "h2d_bytes_per_step": st["h2d_bytes"] / steps_run, "d2h_bytes_per_step": st["d2h_bytes"] / steps_run,
                   "unit_of_work": "one full %d-step run through ffip_create/ffip_run/ffip_output_* "
                                   "(config JSON in from the host, set-up, stepping, DFT arrays out)" % steps_run,
                   "seconds": dt}
        if cs:
            cs.stop()
            cs.__exit__(None, None, None)
            clocks = cs.summary((ta, tb))
    if a.fp32_only:
        res["fp64"] = res["fp32"]
    t32 = res["fp32"]["ms"] / a.steps
    t64 = res["fp64"]["ms"] / a.steps
    value = world * cells / (t32 * 1e-3) / 1e9
    v64 = world * cells / (t64 * 1e-3) / 1e9
    step_achieved = res["fp32"]["bytes_per_step"] / (t32 * 1e-3) / 1e9
    # the dominant kernel's own figure: one launch of the fused pass covers
    # every cell of one step; its algorithmic bytes are the step's (fields,
    # CPML psi, polarisation state, DFT sums: the pass adds the sums of the
    # monitored points itself), over the pass's device time (events around
    # each pass on the stepper's stream)
    tp32 = res["fp32"]["pass_ms"] / a.steps
    if res["fp32"]["fused"] and tp32 > 0:
        achieved = res["fp32"]["bytes_per_step"] / (tp32 * 1e-3) / 1e9
    else:
        tp32 = t32
        achieved = step_achieved

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": warm,
           "ms_per_step": t32, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded spheres, no dataset)", "config": cfg_meta,
           "gpu_launches": res["fp32"]["launches"],
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": profiled_traffic(a.n) if res["fp32"]["fused"] else None,
                        "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one step's k_fused launches "
                                          "(both instances), profiles/k_fused_fp32_dispersive%d.md" % a.n, "peak_kind": peak_kind,
                        "kernel": ("k_fused (both instances, with the face-layer kernels that run beside them)"
                                   if res["fp32"]["fused"] else "k_update (H and E launches)"),
                        "algorithmic_bytes_per_launch": res["fp32"]["bytes_per_step"],
                        "launch_ms": tp32,
                        "timing": "CUDA events on the stepper's stream around each of the %d timed passes (from the first "
                                  "k_fused instance's launch to the join of both); the step's other kernels run inside "
                                  "that window on the side streams" % a.steps,
                        "without_dft": {"algorithmic_bytes": res["fp32"]["pass_bytes_per_step"],
                                        "achieved": res["fp32"]["pass_bytes_per_step"] / (tp32 * 1e-3) / 1e9},
                        "step": {"ms": t32, "achieved": step_achieved, "frac": step_achieved / peak}},
           "fp64": {"value": v64, "unit": UNIT, "ms_per_step": t64, "fp32_speedup": t64 / t32,
                    "achieved_gbs": res["fp64"]["bytes_per_step"] / (t64 * 1e-3) / 1e9,
                    "pass_ms": res["fp64"]["pass_ms"] / a.steps},
           "clocks": clocks}

    # ---- full runs: end to end through the C ABI (fp32, run above inside the
    #      clock window) and the fp32-vs-fp64 DFT error
    if not a.skip_full_run:
        out["e2e"] = e2e
        if not a.fp32_only:
            full["fp64"] = full_run("fp64")[0]
            out["dft_rel_err_fp32_vs_fp64"] = dft_rel_err(full["fp32"], full["fp64"])

    # ---- the plain fp64 vacuum box, GPU beside the CPU restatement
    if not a.fp32_only:
        out["vacuum64_fp64"] = vacuum64_leg(dev, rank == 0 and world == 1 and not a.no_cpu)

    # ---- design iterations of the adjoint workload (forward + one adjoint
    #      run per frequency + gradient), simulations kept between iterations
    if a.design_iters > 0 and not a.fp32_only:
        out["design_iter"] = design_leg(a.design_iters, dev, world)
    if not a.fp32_only:
        try:
            out["set_density"] = set_density_leg(dev)
        except Exception as e:  # reported, not fatal
            out["set_density"] = {"error": str(e)[:300]}
    if not a.no_large and not a.fp32_only:
        try:
            out["large_design"] = large_leg(dev)
        except Exception as e:  # reported, not fatal: the headline line stands without it
            out["large_design"] = {"error": str(e)[:300]}

    # ---- CPU baseline sample (rank 0 only)
    if rank == 0 and world == 1 and not a.no_cpu:
        threads = os.cpu_count() or 1
        try:
            dt, setup = cpu_leg(workloads.dispersive_spheres(n, precision="fp64"), a.cpu_steps, 2, threads)
            out["cpu_baseline"] = {"value": cells * a.cpu_steps / dt / 1e9, "unit": UNIT, "cores": threads,
                                   "cpu_model": cpu_model(), "kind": "port",
                                   "sample": "%d time steps of the full workload after 2 warm-up steps, set-up (%.1f s) untimed"
                                             % (a.cpu_steps, setup)}
        except Exception as e:  # the baseline is reported, not required
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": threads, "kind": "port", "error": str(e)}
    if rank == 0:
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
