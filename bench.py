#!/usr/bin/env python3
"""Benchmark of the cajitafluids per-timestep hot path on GB300.

Workload (one step = Solver::step: advect q/u/v, inputs, pressure projection):
  4096^2 periodic, seeded spectral velocity (rms |u| = 1, k <= 64) and
  scalar, cubic interpolation, dt = 0.5 dx / max|u|, projection to
  ||div u||_L2 <= 1e-8 (FP64 residual), mixed precision (FP32 advection and
  inner PCG, FP64 outer refinement), PCG preconditioned by "PFMG" (the
  reference CLI's default pairing, served by the geometric multigrid
  V-cycle; --precon Diagonal selects Jacobi-PCG).  The same steps in plain
  FP64 are timed for the mixed-vs-FP64 ratio, and the scalar error of the
  mixed run against the FP64 run is reported.

Output: one JSON line (rank 0).  value = steps/s of the mixed form over all
ranks (each rank runs an independent replica; the path is single-GPU).
--impl reference times the reference algorithm's CPU implementation (the
oracle port, all host threads) on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "steps/s at 4096² mixed-prec vs FP64 at ‖div u‖≤1e-8; adjoint/forward ratio"
# bytes the inner Jacobi-PCG kernels of this build move per cell per
# iteration (mixed: K1 R r, p, W p at 4 B; K2 R p, r, W r at 4 B, R/W the
# double-float x at 8 B)
KERNEL_BYTES_MIXED_ITER = 40.0
# Jacobi-PCG iterations per step of this workload in FP64 (the FP64 GPU path
# and the CPU oracle are bit-identical, so they take the same count); with
# --precon Diagonal the reference arm extrapolates its sampled CG cost to this
# count.  Measured by this bench's FP64 leg on GB300.
FP64_ITERS_PER_STEP_4096 = 7890
MG_NAMES = ("PFMG", "SMG", "MG")
# DRAM bytes (read + write) of one mixed MG-PCG inner iteration at 4096^2:
# dram__bytes_read.sum + dram__bytes_write.sum of this bench's kernels, one
# kernel per ncu capture (K1, the fused x update and reliable update, the
# V-cycle's pre- and post-smoothing per level, the bottom solve), summed over
# one iteration
MEASURED_TRAFFIC_MG_ITER_4096 = 1.234e9


def mg_levels(nx, ny, periodic):
    """Level extents of the multigrid hierarchy (the library's coarsening
    rule: halve while both axes are even and >= 16 and the halved extent
    stays even along periodic axes)."""
    lv = [(nx, ny)]
    while not (nx % 2 or ny % 2 or nx < 16 or ny < 16 or (periodic[0] and (nx // 2) % 2)
               or (periodic[1] and (ny // 2) % 2)):
        nx //= 2
        ny //= 2
        lv.append((nx, ny))
    return lv


def alg_bytes_per_iter(nx, ny, periodic, precon, word, outer_frac=0.0, mixed=False):
    """Algorithmic (minimal compulsory) bytes of one PCG iteration, per the
    stage table of the measurement plan (full-grid arrays of `word` bytes,
    ghosts ignored).

    Jacobi: 11 arrays per cell (SpMV + dot: R p, W Ap; update + dot: R x, p,
    r, Ap, W x, r; direction: R r, p, W p; M^-1 from wall flags).
    MG: direction + SpMV (R z, p, W p) 3, update (R p, r, x, W r, x) 5, and
    per V-cycle level above the coarsest 5.5 arrays of that level's cells
    (pre-smoothing: R b, W x, W coarse b at 1/4; post-smoothing: R b, x,
    coarse x at 1/4, W x), the coarsest level 2; FP64 adds r.z (R r, z) 2,
    mixed forms r.z with the finest post-smoothing.  Mixed: the solution x
    is a double-float pair (8 bytes) in the update, and the reliable update
    (R x, b at 8 bytes, W r at 4 = 20 B per cell) runs on the fraction
    outer_frac of the iterations; when that is every iteration, the update
    replaces r, and the x update and the reliable update are one pass
    (R p, x, b, W x, r: 32 B per cell)."""
    n = nx * ny
    if precon not in MG_NAMES:
        return 11 * word * n + outer_frac * 20.0 * n
    xw = 8 if mixed else word
    b = 3 * word * n
    if mixed and outer_frac >= 1.0:
        # x update fused with the reliable update that replaces r
        b += (2 * word + 3 * xw) * n
        outer_frac = 0.0
    else:
        b += (3 * word + 2 * xw) * n
    if not mixed:
        b += 2 * word * n
    lv = mg_levels(nx, ny, periodic)
    for a, c in lv[:-1]:
        b += 5.5 * word * a * c
    b += 2 * word * lv[-1][0] * lv[-1][1]
    return b + outer_frac * 20.0 * n


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_context(w, precision, device):
    from cajitafluids_gb300 import Context
    c = Context(w.nx, w.ny, periodic=w.periodic, precision=precision, device=device)
    c.set_bc(w.bc)
    if w.source is not None:
        c.set_source(*w.source, mode=w.source_mode)
    c.set_body_force(w.body, w.body_density_scaled)
    c.set_density(w.density)
    c.upload("q", w.q0)
    c.upload("u", w.u0)
    c.upload("v", w.v0)
    return c


# Mixed MG-PCG reliable-update threshold of this workload: 0.5, i.e. a
# double-float residual after every iteration (each cuts the residual by more
# than half): 5 iterations and 5 updates per step at 4096^2 instead of 6 and 4
# with the library's default 0.1 (4.08 vs 4.38 ms per step, GB300).
MG_INNER_TOL = 0.5


def solver_opts(w):
    from cajitafluids_gb300 import SolverOptions
    inner = MG_INNER_TOL if w.precon in MG_NAMES else 0.0
    return SolverOptions(tol=w.tol, abs_tol=w.abs_tol, max_iter=w.max_iter, precon=w.precon, inner_tol=inner)


def run_steps(c, w, n, stats=None):
    o = solver_opts(w)
    for _ in range(n):
        s = c.step(w.dt, w.order, o, raise_on_maxit=True)
        if stats is not None:
            stats.append(s)


def barrier_sync(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# --------------------------------------------------------------------------
def cpu_reference_sample(w, k_iters, m1=5, m2=15, steps=1):
    """Oracle (CPU port of the reference algorithm, all OpenMP threads) timed
    on a bounded sample of the workload.  MG-PCG: whole steps (one untimed
    first).  Jacobi-PCG: one advection + inputs, and the projection capped at
    m1 and m2 CG iterations; the CG cost per iteration and the fixed
    projection cost are extrapolated to k_iters iterations."""
    from oracle import Oracle, threads
    mg = w.precon in MG_NAMES
    o = Oracle(w.nx, w.ny, periodic=w.periodic, bc=w.bc, source=w.source, source_mode=w.source_mode,
               body=w.body, body_density_scaled=w.body_density_scaled, density=w.density, precon_mg=mg)
    o.set("q", w.q0)
    o.set("u", w.u0)
    o.set("v", w.v0)
    per_step = []
    detail = {}
    if mg:
        iters = []
        for s in range(steps + 1):
            t0 = time.perf_counter()
            st = o.step(w.dt, w.order, tol=w.tol, abs_tol=w.abs_tol, max_iter=w.max_iter)
            if s > 0:
                per_step.append(time.perf_counter() - t0)
                iters.append(st["iterations"])
        detail = {"mg_iters_per_step": statistics.mean(iters), "sample_steps": steps,
                  "sampled_wall_s": sum(per_step)}
        return per_step, threads(), detail
    for _ in range(steps):
        t0 = time.perf_counter()
        o.advect(w.dt, w.order)
        o.add_inputs(w.dt)
        t1 = time.perf_counter()
        snap = {f: o.get(f) for f in ("u", "v")}
        o.project(w.dt, tol=w.tol, abs_tol=w.abs_tol, max_iter=m1)
        t2 = time.perf_counter()
        o.set("u", snap["u"])
        o.set("v", snap["v"])
        o.project(w.dt, tol=w.tol, abs_tol=w.abs_tol, max_iter=m2)
        t3 = time.perf_counter()
        t_iter = max((t3 - t2) - (t2 - t1), 0.0) / (m2 - m1)
        t_fixed = max((t2 - t1) - m1 * t_iter, 0.0)
        t_step = (t1 - t0) + t_fixed + k_iters * t_iter
        per_step.append(t_step)
        detail = {"advect_inputs_s": t1 - t0, "cg_iter_s": t_iter, "projection_fixed_s": t_fixed,
                  "sampled_wall_s": t3 - t0}
    return per_step, threads(), detail


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


# --------------------------------------------------------------------------
def bench_gb300(args, rank, world, dist, device):
    from cajitafluids_gb300.workloads import config2
    t_gen = time.perf_counter()
    w = config2(args.size, steps=args.steps)
    w.precon = args.precon
    mg = w.precon in MG_NAMES
    w.max_iter = 2000 if mg else 400000
    t_gen = time.perf_counter() - t_gen
    ncell = w.nx * w.ny
    pc_text = "PCG + PFMG-named geometric multigrid V-cycle" if mg else f"PCG + {w.precon}"

    legs = set(args.legs.split(","))
    peak, peak_kind = measured_peaks()
    line = {
        "metric": METRIC, "value": None, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic: seeded spectral velocity (k<=64, per-mode power k^-11/3, rms|u|=1) and scalar",
        "config": {"workload": f"{w.nx}x{w.ny} periodic spectral, mixed precision (FP32 advection + inner PCG, "
                               f"FP64 outer refinement), cubic, {pc_text}, ||div u||_L2 <= {w.abs_tol:g}",
                   "nx": w.nx, "ny": w.ny, "periodic": True, "precision": "mixed", "value_order": w.order,
                   "dt": w.dt, "abs_tol_div_l2": w.abs_tol, "solver": "PCG", "precon": w.precon,
                   "reliable_update_threshold": solver_opts(w).inner_tol or 0.1,
                   "mg_levels": len(mg_levels(w.nx, w.ny, w.periodic)) if mg else None,
                   "parallelism": f"replicas x{world}",
                   "l2_policy": "inputs larger than L2 (state + solver vectors ~1 GB)"},
        "adjoint_forward_ratio": None,
    }
    value = None
    stats = []
    if "mixed" in legs:
        # ---- mixed precision (headline) ----
        cm = make_context(w, "mixed", device)
        run_steps(cm, w, args.warmup)
        l0 = cm.launches
        clocks = ClockSampler(device)
        barrier_sync(dist)
        cm.timer_start()
        t_wall = time.perf_counter()
        clocks.start()
        # Solver::solve's loop on the device (cf_steps): the steps go back to
        # back, one synchronisation; it raises if any step's solve did not
        # converge
        last = cm.steps(args.steps, w.dt, w.order, solver_opts(w), raise_on_maxit=True)
        ms = cm.timer_stop()
        clk = clocks.stop()
        t_wall = time.perf_counter() - t_wall
        launches = cm.launches - l0
        stats.append(last)
        # a profiled pass after the timed one (per-step statistics): with
        # profiling on, the projection runs host-polled graph batches with
        # CUDA events around them (the timed steps run one device-resident
        # graph per projection)
        cm.profile_enable(True)
        run_steps(cm, w, min(args.steps, 10), stats)
        prof = cm.profile_read()
        cm.profile_enable(False)
        ms_max = max_over_ranks(dist, ms)
        value = world * args.steps / (ms_max / 1e3)
        it_ms = prof["solve_ms"] / prof["solve_iters"] if prof["solve_iters"] else float("nan")
        iters = statistics.mean(s["iterations"] for s in stats)
        outers = statistics.mean(s["outer_iterations"] for s in stats)
        it_bytes = alg_bytes_per_iter(w.nx, w.ny, w.periodic, w.precon, 4, min(outers / max(iters, 1), 1.0),
                                      mixed=True)
        achieved = it_bytes / (it_ms / 1e3) / 1e9
        if mg:
            kname = ("MG-PCG inner iteration: k_tma_dir_matvec32 + k_outer_resid<true> (x update fused with the "
                     "reliable update; at an update threshold below 0.5, k_tma_update32 + gated k_outer_resid) + "
                     "V-cycle (k_mg_pre/k_mg_post per level with r.z in the finest post-smoothing, k_mg_bottom)")
            kern_extra = {}
        else:
            kname = "inner CG iteration (k_tma_dir_matvec32 + k_tma_update32)"
            kern_extra = {"kernel_bytes_per_cell": KERNEL_BYTES_MIXED_ITER,
                          "kernel_bytes_gbs": KERNEL_BYTES_MIXED_ITER * ncell / (it_ms / 1e3) / 1e9}
        line.update({
            "value": value, "ms_per_step": ms_max / args.steps, "cell_updates_per_s": value * ncell,
            "mixed": {"cg_inner_iters_per_step": iters, "outer_refinements_per_step": outers,
                      "stats_steps": "the timed run's last step and the 10 profiled steps after it; "
                                     "every timed step's solve converged (cf_steps counts the others)",
                      "timed_unconverged": last["unconverged"],
                      "div_l2_max": max(s["div_l2"] for s in stats),
                      "div_linf_max": max(s["div_linf"] for s in stats),
                      "advect_ms_per_step": prof["advect_ms"] / max(prof["advect_calls"], 1),
                      "cg_iter_ms": it_ms, "cg_iters_timed": prof["solve_iters"],
                      "project_ms_per_step": prof["project_ms"] / max(prof["projects"], 1)},
            "roofline": {"bound": "hbm", "kernel": kname,
                         "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": f"hbm_gbs {peak_kind}",
                         "traffic": MEASURED_TRAFFIC_MG_ITER_4096 if (mg and w.nx == 4096) else None,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one kernel per "
                                           "capture, summed over the kernels of one inner iteration"
                                           if (mg and w.nx == 4096) else None,
                         "algorithmic_bytes": it_bytes,
                         "algorithmic_bytes_per_cell": it_bytes / ncell, **kern_extra},
            "gpu_launches": launches, "clocks": clk,
            "timing": {"device_ms": ms, "wall_s": t_wall, "workload_gen_s": t_gen},
        })

        if "e2e" in legs:
            # ---- e2e through the C ABI with host buffers ----
            from cajitafluids_gb300.api import PinnedArray
            hq = PinnedArray(cm.owned_shape("q"))
            hu = PinnedArray(cm.owned_shape("u"))
            hv = PinnedArray(cm.owned_shape("v"))
            for h, f in ((hq, "q"), (hu, "u"), (hv, "v")):
                cm.download(f, h.array)
            o = solver_opts(w)
            e2e_steps = max(1, args.e2e_steps)
            # warm-up calls: the first one creates the second stream, the
            # events and the quantity's download staging (made on first use)
            for _ in range(max(1, args.warmup)):
                cm.step_host(w.dt, w.order, o, hq.array, hu.array, hv.array, hq.array, hu.array, hv.array,
                             raise_on_maxit=True)
            barrier_sync(dist)
            cm.timer_start()
            t_e2e = time.perf_counter()
            for _ in range(e2e_steps):
                # upload q, u, v from page-locked host memory, step, download
                # them again: one C-ABI call per step (cf_step_host)
                cm.step_host(w.dt, w.order, o, hq.array, hu.array, hv.array, hq.array, hu.array, hv.array,
                             raise_on_maxit=True)
            e2e_ms = cm.timer_stop()
            t_e2e = time.perf_counter() - t_e2e
            e2e_ms = max_over_ranks(dist, max(e2e_ms, t_e2e * 1e3))
            io_bytes = 8 * (hq.array.size + hu.array.size + hv.array.size)
            line["e2e"] = {"value": world * e2e_steps / (e2e_ms / 1e3), "unit": "steps/s",
                           "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes,
                           "path": "cf_step_host: q,u,v from pinned host, one step, q,u,v back to pinned host "
                                   "(q's upload overlaps the u,v advection, q's download the projection, "
                                   "u,v's download the step's tail; on this periodic grid the divergence norms are taken "
                                   "inside the gradient kernel, before u,v go out)"}
            for h in (hq, hu, hv):
                h.free()
        cm.close()

    if "warm" in legs and "mixed" in legs:
        # the same workload with warm-started projections (extension; the
        # reference cold-starts): steps/s and iterations per step
        cw = make_context(w, "mixed", device)
        cw.set_warm_start(True)
        run_steps(cw, w, args.warmup)
        wst = []
        nwarm = min(args.steps, 100)
        cw.timer_start()
        run_steps(cw, w, nwarm, wst)
        msw = cw.timer_stop()
        cw.close()
        line["warm_start"] = {"steps_per_s": nwarm / (msw / 1e3),
                              "cg_inner_iters_per_step": statistics.mean(s["iterations"] for s in wst),
                              "outer_refinements_per_step": statistics.mean(s["outer_iterations"] for s in wst),
                              "div_l2_max": max(s["div_l2"] for s in wst), "steps": nwarm}

    fstats = []
    k64 = None
    if "fp64" in legs:
        # ---- plain FP64 on the same steps ----
        cf = make_context(w, "fp64", device)
        run_steps(cf, w, args.warmup, fstats)
        barrier_sync(dist)
        cf.timer_start()
        run_steps(cf, w, args.fp64_steps, fstats)
        ms64 = cf.timer_stop()
        cf.profile_enable(True)
        run_steps(cf, w, min(args.fp64_steps, 4))
        prof64 = cf.profile_read()
        cf.close()
        ms64 = max_over_ranks(dist, ms64)
        value64 = world * args.fp64_steps / (ms64 / 1e3) if args.fp64_steps else None
        k64 = statistics.mean(s["iterations"] for s in fstats[args.warmup:]) if args.fp64_steps else None
        it64_ms = prof64["solve_ms"] / prof64["solve_iters"] if prof64["solve_iters"] else float("nan")
        achieved64 = alg_bytes_per_iter(w.nx, w.ny, w.periodic, w.precon, 8) / (it64_ms / 1e3) / 1e9
        line["fp64"] = {"steps_per_s": value64, "cg_iters_per_step": k64, "cg_iter_ms": it64_ms,
                        "advect_ms_per_step": prof64["advect_ms"] / max(prof64["advect_calls"], 1),
                        "project_ms_per_step": prof64["project_ms"] / max(prof64["projects"], 1),
                        "roofline_hbm_frac": achieved64 / peak,
                        "div_l2_max": max(s["div_l2"] for s in fstats) if fstats else None}
        if value and value64:
            line["mixed_vs_fp64"] = value / value64

    if "accuracy" in legs:
        line["scalar_error_vs_fp64"] = bench_accuracy(args, w, device)

    if "configs" in legs:
        line["configs_0_1"] = bench_configs(args, device)

    if "adjoint" in legs:
        line["adjoint"] = bench_adjoint(args, device, dist)
        line["adjoint_forward_ratio"] = line["adjoint"]["forward_plus_adjoint_over_forward"]

    if "adjoint4" in legs:
        line["adjoint_mixed"] = bench_adjoint4(args, device, dist, peak)

    # ---- CPU baseline (rank 0, N = 1) ----
    if rank == 0 and world == 1 and "cpu" in legs and not args.skip_cpu:
        k_ref = k64 if k64 else (line.get("mixed", {}).get("cg_inner_iters_per_step") or args.ref_iters)
        per_step, cores, detail = cpu_reference_sample(w, k_ref, steps=2 if mg else 1)
        if mg:
            sample = (f"oracle FP64 MG-PCG on the same {w.nx}^2 state: 2 whole steps timed after 1 untimed "
                      f"(advection + inputs + projection to the same tolerance)")
        else:
            sample = (f"oracle FP64 on the same {w.nx}^2 state: 1 advection+inputs and the projection capped "
                      f"at 5 and 15 CG iterations, extrapolated to {k_ref:.0f} iterations/step")
        line["cpu_baseline"] = {"value": 1.0 / statistics.mean(per_step), "unit": "steps/s", "cores": cores,
                                "kind": "port", "cpu": cpu_model(), "sample": sample, **detail}
    return line


def bench_accuracy(args, w, device):
    """The workload's full run (config 2: 200 steps) in mixed precision and
    in FP64 from the same initial state: the scalar's L-inf and RMS error
    of the mixed run against the FP64 run every 20 steps, and the largest
    ||div u||_L2 after any projection of either run."""
    n = max(1, args.accuracy_steps)
    cm = make_context(w, "mixed", device)
    cf = make_context(w, "fp64", device)
    o = solver_opts(w)
    every = []
    div_m, div_f = 0.0, 0.0
    for s in range(1, n + 1):
        div_m = max(div_m, cm.step(w.dt, w.order, o, raise_on_maxit=True)["div_l2"])
        div_f = max(div_f, cf.step(w.dt, w.order, o, raise_on_maxit=True)["div_l2"])
        if s % 20 == 0 or s == n:
            err = cm.download("q") - cf.download("q")
            every.append({"step": s, "linf": float(np.abs(err).max()), "l2": float(np.sqrt(np.mean(err * err)))})
    cm.close()
    cf.close()
    last = every[-1]
    return {"after_steps": n, "linf": last["linf"], "l2": last["l2"], "target_linf": 1e-6,
            "meets_target": last["linf"] <= 1e-6, "every_20_steps": every,
            "div_l2_max_mixed": div_m, "div_l2_max_fp64": div_f,
            "run": f"{w.nx}^2 from the workload's initial state, {n} steps each, mixed and FP64"}


def bench_configs(args, device):
    """Configs 0 and 1 of the benchmark plan at full size and length, FP64,
    Jacobi-PCG (the reference's own solver form), one cf_step per step:
    steps/s, CG iterations per step and ||div u||_L2 after every projection
    (setup's included).  Their fields equal the oracle's bit for bit (the
    GPU tests check all 100 steps of config 0 and the first two of config
    1); here they are only run and measured."""
    from cajitafluids_gb300 import Context, SolverOptions
    from cajitafluids_gb300.workloads import config0, config1
    out = {}
    for name, w, max_iter in (("config0", config0(), 20000), ("config1", config1(), 50000)):
        c = Context(w.nx, w.ny)
        c.set_bc(w.bc)
        c.set_source(*w.source, mode=w.source_mode)
        c.set_body_force(w.body, w.body_density_scaled)
        c.set_density(w.density)
        o = SolverOptions(tol=w.tol, max_iter=max_iter, precon="Diagonal")
        st = [c.setup(w.dt, o, raise_on_maxit=True)]
        c.timer_start()
        t0 = time.perf_counter()
        for _ in range(w.steps):
            st.append(c.step(w.dt, w.order, o, raise_on_maxit=True))
        ms = c.timer_stop()
        wall = time.perf_counter() - t0
        c.close()
        div = [s["div_l2"] for s in st]
        out[name] = {"workload": f"{w.nx}^2 walls, inflow, " + ("gravity scaled by the quantity, " if w.body_density_scaled
                                                                  else "") +
                                 f"{'cubic' if w.order == 3 else 'linear'} values, FP64 PCG + Diagonal to {w.tol:g}, "
                                 f"setup + {w.steps} steps",
                     "steps": w.steps, "steps_per_s": w.steps / (max(ms, wall * 1e3) / 1e3),
                     "cg_iters_per_step": statistics.mean(s["iterations"] for s in st[1:]),
                     "all_converged": all(s["status"] == 0 for s in st),
                     "div_l2_max": max(div), "div_l2_last": div[-1],
                     "div_l2_every_projection": [float(f"{d:.3g}") for d in div]}
    return out


def bench_adjoint(args, device, dist):
    """Forward + adjoint on the 512^2 walls problem with 8 Gaussian blobs:
    loss = 1/2 |q(T) - target|^2, gradient with respect to q(0), u(0), v(0)
    and the rate of a rate-form inflow, T steps, checkpoint every 14."""
    from cajitafluids_gb300 import Context, SolverOptions
    from cajitafluids_gb300 import _lib as L
    from cajitafluids_gb300.workloads import config3
    w = config3(args.adjoint_size, steps=args.adjoint_steps)
    every = args.adjoint_every
    mg = args.precon in MG_NAMES
    opts = SolverOptions(tol=w.tol, max_iter=2000 if mg else 200000, precon=args.precon)
    inflow = ((0.45, 0.10), (0.10, 0.05), (0.0, 0.0), 1.0)

    def fresh(rate=1.0):
        c = Context(w.nx, w.ny, device=device)
        c.set_density(w.density)
        c.set_quirks(L.CF_FIX_Q1)
        c.set_source(inflow[0], inflow[1], inflow[2], rate, mode=1)
        for f, a in (("q", w.q0), ("u", w.u0), ("v", w.v0)):
            c.upload(f, a)
        return c

    c = fresh()
    c.step(w.dt, w.order, opts)  # warm the graphs
    c.close()
    # the plain forward: Solver::solve's loop on the device (cf_steps), the
    # fastest forward this build has, so the ratio is against it
    c = fresh()
    barrier_sync(dist)
    c.timer_start()
    last = c.steps(w.steps, w.dt, w.order, opts, raise_on_maxit=True)
    t_fwd = c.timer_stop()
    qT = c.download("q")
    c.close()
    c = fresh()
    its = sum(c.step(w.dt, w.order, opts)["iterations"] for _ in range(min(w.steps, 20)))
    its_steps = min(w.steps, 20)
    c.close()
    c = fresh()
    c.timer_start()
    c.forward_checkpointed(w.steps, every, w.dt, w.order, opts)
    t_fc = c.timer_stop()
    target = w.extra["target"]
    c.timer_start()
    g = c.backward(c.download("q") - target)
    t_bwd = c.timer_stop()
    assert np.array_equal(c.download("q"), qT)   # checkpointed forward = plain forward
    out = {"workload": f"{w.nx}^2 walls, spectral velocity + 8 Gaussian blobs, rate inflow, T={w.steps}, "
                       f"checkpoint every {every}, FP64, PCG + {args.precon}, tol {w.tol:g}",
           "forward_ms": t_fwd, "forward_checkpointed_ms": t_fc, "backward_ms": t_bwd,
           "forward_plus_adjoint_over_forward": (t_fc + t_bwd) / t_fwd,
           "cg_iters_per_forward_step": its / its_steps, "forward_unconverged": last["unconverged"],
           "loss": 0.5 * float(np.sum((qT - target) ** 2))}
    # central differences of the FP64 forward on seeded directions
    rng = np.random.default_rng(16)
    checks = []
    for k in range(args.adjoint_fd):
        dq = rng.standard_normal(w.q0.shape)
        du = rng.standard_normal(w.u0.shape)
        dv = rng.standard_normal(w.v0.shape)
        du[:, 0] = du[:, -1] = 0.0
        dv[0, :] = dv[-1, :] = 0.0
        h = 1e-6
        vals = []
        for sgn in (1.0, -1.0):
            c2 = fresh()
            for f, a, d in (("q", w.q0, dq), ("u", w.u0, du), ("v", w.v0, dv)):
                c2.upload(f, a + sgn * h * d)
            for _ in range(w.steps):
                c2.step(w.dt, w.order, opts)
            vals.append(0.5 * float(np.sum((c2.download("q") - target) ** 2)))
            c2.close()
        fd = (vals[0] - vals[1]) / (2 * h)
        ad = float(np.sum(g["q"] * dq) + np.sum(g["u"] * du) + np.sum(g["v"] * dv))
        checks.append({"fd": fd, "adjoint": ad, "rel_err": abs(fd - ad) / max(abs(ad), 1e-300)})
    out["fd_checks"] = checks
    out["dL_drate"] = g["rate"]
    c.close()
    return out


def mixed_state_bytes(n):
    """Bytes of one checkpointed mixed state at n^2 with walls: the ghosted
    FP32 q and the u, v pair arrays as the library lays them out (rows padded
    so that owned column 0 sits on a 128-byte boundary)."""
    def pitch(ex):
        return (29 + ex + 31) // 32 * 32
    return pitch(n + 6) * (n + 6) * 4 + pitch(n + 7) * (n + 6) * 8 + pitch(n + 6) * (n + 7) * 8


def bench_adjoint4(args, device, dist, peak):
    """Config 4: mixed-precision forward + adjoint at 8192^2 with walls,
    cubic values, seeded spectral velocity and scalar, ||div u||_L2 <= 1e-8,
    T steps with a checkpoint every sqrt(T).  Timed after one warm-up
    forward/backward on the same context (graphs built), from the initial
    state re-uploaded.  Per-kernel rates come from a short profiled run of
    the same context (events around each stage)."""
    from cajitafluids_gb300 import Context, SolverOptions
    from cajitafluids_gb300 import _lib as L
    from cajitafluids_gb300.workloads import config4
    t0 = time.perf_counter()
    n, T = args.adjoint4_size, args.adjoint4_steps
    w = config4(n, steps=T)
    t_gen = time.perf_counter() - t0
    sq = max(1, int(round(math.sqrt(T))))
    sb = mixed_state_bytes(n)

    def fits(C):
        return ((T + C - 1) // C + C + 1) * sb <= 150e9

    # checkpoints sized to the 150 GB budget with recomputation between them:
    # the smallest spacing >= 2 that fits; the sqrt(T) spacing is timed too
    every = args.adjoint4_every or next((C for C in range(2, T + 1) if fits(C)), sq)
    mg = args.precon in MG_NAMES
    opts = SolverOptions(tol=0.0, abs_tol=w.abs_tol, max_iter=2000 if mg else 200000, precon=args.precon,
                         inner_tol=0.5 if mg else 0.0)
    target = w.extra["target"]

    def load(c):
        for f, a in (("q", w.q0), ("u", w.u0), ("v", w.v0)):
            c.upload(f, a)

    def fresh():
        c = Context(n, n, precision="mixed", device=device)
        c.set_density(w.density)
        c.set_quirks(L.CF_FIX_Q1)
        load(c)
        return c

    # plain forward (cf_steps), after one warm-up step
    c = fresh()
    c.step(w.dt, w.order, opts)
    load(c)
    barrier_sync(dist)
    c.timer_start()
    last = c.steps(T, w.dt, w.order, opts, raise_on_maxit=True)
    t_fwd = c.timer_stop()
    qT = c.download("q")
    c.close()
    # checkpointed forward + backward, after a 2-step warm-up of both
    c = fresh()
    c.forward_checkpointed(2, 1, w.dt, w.order, opts)
    c.backward(np.zeros_like(w.q0))
    runs = {}
    for C in dict.fromkeys((every, sq)):
        load(c)
        c.timer_start()
        st = c.forward_checkpointed(T, C, w.dt, w.order, opts)
        t_fc = c.timer_stop()
        q_fc = c.download("q")
        c.timer_start()
        g = c.backward(q_fc - target)
        t_bwd = c.timer_stop()
        runs[C] = {"every": C, "checkpoint_gb": ((T + C - 1) // C + C + 1) * sb / 1e9,
                   "forward_checkpointed_ms": t_fc, "backward_ms": t_bwd,
                   "forward_plus_adjoint_over_forward": (t_fc + t_bwd) / t_fwd,
                   "checkpointed_forward_equals_plain": bool(np.array_equal(q_fc, qT))}
        if C == every:
            g_main, st_main, q_main = g, st, q_fc
    g, st, q_fc = g_main, st_main, q_main
    # per-kernel rates (profiled run: host-polled projections, events around
    # each stage; 4 steps, checkpoint every 2)
    load(c)
    c.profile_enable(True)
    c.forward_checkpointed(4, 2, w.dt, w.order, opts)
    c.backward(c.download("q") - target)
    prof = c.profile_read()
    c.profile_enable(False)
    c.close()
    ncell = n * n
    adv_ms = prof["advect_ms"] / max(prof["advect_calls"], 1)
    radv_ms = prof["adj_advect_ms"] / max(prof["adj_advect_calls"], 1)
    it_ms = prof["solve_ms"] / prof["solve_iters"] if prof["solve_iters"] else float("nan")
    it_bytes = alg_bytes_per_iter(n, n, (False, False), args.precon, 4, 1.0, mixed=True)
    # bytes per cell: advection R q 4 + u, v pairs 16, W the same (40); reverse
    # advection R forward q 4 + u, v pairs 16, R adjoint q 4 + u, v pairs 16,
    # W the three FP32 outputs 12 (52)
    kern = {"advect32": {"ms": adv_ms, "bytes_per_cell": 40,
                         "gbs": 40 * ncell / (adv_ms / 1e3) / 1e9 if adv_ms else None},
            "adj_advect32": {"ms": radv_ms, "bytes_per_cell": 52,
                             "gbs": 52 * ncell / (radv_ms / 1e3) / 1e9 if radv_ms else None},
            "mg_pcg_iteration": {"ms": it_ms, "bytes": it_bytes,
                                 "gbs": it_bytes / (it_ms / 1e3) / 1e9 if it_ms == it_ms else None}}
    for k in kern.values():
        if k.get("gbs"):
            k["hbm_frac"] = k["gbs"] / peak
    main = runs[every]
    return {"workload": f"{n}^2 walls, cubic, seeded spectral velocity + scalar, T={T}, checkpoint every {every} "
                        f"(the smallest spacing whose checkpoints fit 150 GB), mixed precision (FP32 bulk, "
                        f"double-float refinement), PCG + {args.precon}, ||div u||_L2 <= {w.abs_tol:g}; adjoint: "
                        f"FP32 reverse advection, transposed projection to relative 1e-7 (warm-started)",
            "forward_ms": t_fwd, "forward_steps_per_s": T / (t_fwd / 1e3),
            **main,
            "sqrt_spacing": runs[sq],
            "adjoint_cg_iters_per_projection": prof["adj_iters"] / max(prof["adj_projects"], 1),
            "forward_last_step": {"iterations": st["iterations"], "outer_iterations": st["outer_iterations"],
                                  "div_l2": st["div_l2"]},
            "forward_unconverged": last["unconverged"],
            "loss": 0.5 * float(np.sum((q_fc - target) ** 2)),
            "gradient_norms": {f: float(np.linalg.norm(g[f])) for f in ("q", "u", "v")},
            "gradient_finite": bool(all(np.isfinite(g[f]).all() for f in ("q", "u", "v"))),
            "kernels": kern, "workload_gen_s": t_gen}


def bench_reference(args, rank, world, dist):
    """The reference algorithm's CPU implementation (oracle port) on the same
    workload and metric; rank 0 only."""
    if rank != 0:
        return None
    from cajitafluids_gb300.workloads import config2
    w = config2(args.size, steps=args.steps)
    w.precon = args.precon
    mg = w.precon in MG_NAMES
    w.max_iter = 2000 if mg else 400000
    k_ref = FP64_ITERS_PER_STEP_4096 if (FP64_ITERS_PER_STEP_4096 and args.size == 4096) else args.ref_iters
    per = []
    detail = {}
    if mg:
        # whole steps; at 4096^2 one step is a few seconds on 16 cores
        n_steps = max(1, min(args.steps, 3))
        per, cores, detail = cpu_reference_sample(w, k_ref, steps=n_steps)
        sample = f"{n_steps} whole MG-PCG steps after 1 untimed"
    else:
        total = max(1, args.steps) + max(0, min(args.warmup, 1))
        for s in range(total):
            p, cores, detail = cpu_reference_sample(w, k_ref)
            if s >= total - max(1, args.steps):
                per.extend(p)
        sample = (f"per step: 1 advection+inputs and the projection capped at 5 and 15 CG iterations, "
                  f"extrapolated to {k_ref} iterations/step")
    value = 1.0 / statistics.mean(per)
    return {
        "metric": METRIC, "impl": "reference", "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": len(per), "warmup": 1, "ms_per_step": 1e3 * statistics.mean(per),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded spectral velocity (k<=64, per-mode power k^-11/3, rms|u|=1) and scalar",
        "config": {"workload": f"{w.nx}x{w.ny} periodic spectral, FP64 reference algorithm (CPU), cubic, "
                               f"PCG + {w.precon}, ||div u||_L2 <= {w.abs_tol:g}", "nx": w.nx, "ny": w.ny,
                   "precon": w.precon},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": sample, **detail},
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_unbuildable": "Kokkos/Cabana-Cajita/HYPRE/MPI are not available; the oracle is the CPU port",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--size", type=int, default=4096)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--legs", default="mixed,e2e,warm,fp64,accuracy,configs,adjoint,adjoint4,cpu",
                    help="comma list of legs to run: mixed (headline), e2e, warm, fp64, accuracy, configs, "
                         "adjoint (config 3, FP64), adjoint4 (config 4, mixed), cpu")
    ap.add_argument("--accuracy-steps", type=int, default=200,
                    help="steps of the mixed-vs-FP64 accuracy run (the workload's full run length)")
    ap.add_argument("--adjoint-size", type=int, default=512)
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-every", type=int, default=14)
    ap.add_argument("--adjoint-fd", type=int, default=2, help="central-difference checks of the gradient")
    ap.add_argument("--adjoint4-size", type=int, default=8192)
    ap.add_argument("--adjoint4-steps", type=int, default=100)
    ap.add_argument("--adjoint4-every", type=int, default=0, help="checkpoint spacing (0: sqrt of the steps)")
    ap.add_argument("--ref-iters", type=int, default=12000)
    ap.add_argument("--precon", default="PFMG",
                    help="PCG preconditioner: PFMG/SMG/MG (geometric multigrid, the reference CLI default), "
                         "Diagonal (Jacobi) or None")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as td
        backend = "gloo"
        td.init_process_group(backend=backend)
        dist = td
    if args.impl == "reference":
        line = bench_reference(args, rank, world, dist)
    else:
        from __graft_entry__ import build
        build()
        line = bench_gb300(args, rank, world, dist, local)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
