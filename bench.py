"""Benchmark: RS two-phase pressure step on one GB300.

Workload: 3D oil/water black-oil case on a perturbed 128 x 128 x 32 hex grid
(524,288 cells), lognormal permeability (kz/kx = 0.1), Corey n = 2,
Swc = Sor = 0.2, five-spot wells; MPFA-O transmissibilities; every step is
one Discretisation.solve(dt): the pressure Newton loop (properties, Darcy
fluxes, Jacobian assembly, BiCGstab + ILU(0) to 1e-8 relative residual,
pressure update) and the explicit molar-mass update.  The timed steps are
the first K steps from the initial state (the GPU takes its W warm-up steps
first and returns to the initial state).

Metric: cell-Newton-steps/s = cells x pressure Newton iterations / seconds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl resgpu|reference]

Prints one JSON line on rank 0.  `value` is device time (CUDA events on the
library's stream, inputs resident); `e2e` replays the same K steps from the
initial state through the public API with the state staged through
page-locked host memory every step.  `--impl reference` times the CPU oracle
(the C++ restatement of RS + MTJ, single-threaded like RS) on the same K
steps with the same converged Newton loop.

The same line carries the other measured legs as sub-objects: the
mixed-precision solver on the same steps, the Peng-Robinson flash, the
compositional line drive, the discrete adjoint of 50 steps with a checkpoint
every 10, the ensemble of 64 members and the AMG preconditioner; with no
flags the whole run takes about eight minutes on one GB300 (each leg has a
flag to shorten or skip it).
"""
import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from ressim_gb300 import abi  # noqa: E402
from ressim_gb300 import workloads as W  # noqa: E402

METRIC = "cell-Newton-steps/s"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx = max(mx, float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def build_case(args):
    case = W.two_phase_case(ni=args.ni, nj=args.nj, nk=args.nk, seed=args.seed)
    keep = abi.Keep()
    fluid = W.two_phase_fluid(keep)
    co = W.corey()
    srcs = W.build_sources(keep, case)
    init = W.build_initial(case)
    spec = W.runspec(rtol=args.rtol, atol=1e-50)
    return case, keep, fluid, co, srcs, init, spec


# DRAM bytes (read + write) per launch of the ILU(0) level walks, measured by
# one ncu capture of this workload (dram__bytes_read.sum +
# dram__bytes_write.sum); keyed by grid size and kernel family.  ncu cannot
# run inside the timed benchmark, so the line labels these as a capture's.
NCU_TRAFFIC = {(128, 128, 32): {"ilu_lower": 103_740_416, "ilu_upper": 107_909_632}}
NCU_TRAFFIC_SOURCE = "ncu capture of the same kernel on the same workload (not measured in this run)"


def config_of(args, nnz, dt):
    """Workload description shared by both arms (same keys, same values)."""
    return {"workload": f"two-phase oil/water black-oil, {args.ni}x{args.nj}x{args.nk} perturbed hex grid, MPFA-O, "
                        f"BiCGstab+ILU(0) FP64 to {args.rtol:g} relative residual, Newton converged per step, "
                        f"first K steps from the initial state",
            "cells": args.ni * args.nj * args.nk, "pattern_nnz": int(nnz), "dt_s": dt, "seed": args.seed}


def sweep_bytes(rp, col):
    """Algorithmic bytes of one ILU(0) triangular sweep: each strictly
    lower (or upper) coefficient (8 B) and its column index (4 B), the
    right-hand side read and the result written (16 B per row), plus the
    diagonal (8 B per row) for the upper sweep."""
    n = len(rp) - 1
    rows = np.repeat(np.arange(n), np.diff(rp))
    lower = int(np.count_nonzero(col < rows))
    upper = int(np.count_nonzero(col > rows))
    return 12 * lower + 16 * n, 12 * upper + 24 * n


def run_resgpu(args, rank, world, local_rank):
    from ressim_gb300 import api

    case, keep, fluid, co, srcs, init, spec = build_case(args)
    ctx = api.Context(local_rank)
    mesh = api.Mesh(ctx, 3, args.ni, args.nj, args.nk, case["perm"], coords=case["nodes"])
    mesh.compute_mpfa()
    counts = mesh.counts()
    n = counts["elements"]
    sim = api.Discretisation(ctx, mesh, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    dt = case["dt"]
    sim.save_state()  # the initial state: the timed and end-to-end passes both start here
    for _ in range(args.warmup):
        sim.step(dt)
    sim.restore_state()
    barrier(world)
    clocks = ClockSampler(local_rank)
    clocks.start()
    ctx.synchronize()
    launches0 = ctx.kernel_launches()
    newton = 0
    linear = 0
    ctx.timer_record(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        info = sim.step(dt)
        newton += info.newton_iterations
        linear += info.linear_iterations
    ctx.timer_record(1)
    ctx.synchronize()
    wall = time.perf_counter() - t0
    ms = ctx.timer_elapsed_ms(0, 1)
    launches = ctx.kernel_launches() - launches0
    clk = clocks.stop()
    dev_s = ms / 1e3
    dev_s = max_over_ranks(dev_s, world)
    units = float(n) * newton
    units = sum_over_ranks(units, world)
    p_end = sim.state()[0]

    # end to end through the public API with page-locked host staging
    nc = sim.nc
    e2e = None if args.no_e2e else e2e_pass(args, ctx, sim, n, nc, dt, world, newton, p_end)
    res = finish(args, ctx, mesh, sim, n, world, units, dev_s, wall, launches, clk, newton, linear, dt, e2e, rank)
    # the secondary legs report their failure instead of ending the run
    def leg(name, fn):
        try:
            res[name] = fn()
        except Exception as e:  # noqa: BLE001
            res[name] = {"error": f"{type(e).__name__}: {e}"}

    if args.mixed_steps >= 0:
        leg("mixed", lambda: mixed_leg(args, ctx, mesh, case, fluid, co, srcs, init, sim, n, dt, dev_s, p_end, world))
    if args.ensemble > 0 and rank == 0:
        leg("ensemble", lambda: ensemble_leg(args))
    if args.flash_cells > 0 and rank == 0:
        leg("flash", lambda: flash_leg(args))
    if args.comp_steps > 0 and rank == 0:
        leg("compositional", lambda: compositional_leg(args))
    if args.adj_steps > 0:
        leg("adjoint", lambda: adjoint_leg(args, ctx, mesh, case, fluid, co, srcs, init, n, world))
    if args.amg and rank == 0:
        leg("amg", lambda: amg_leg(args, ctx, mesh, case, fluid, co, srcs, init, n, world))
    return res


def e2e_pass(args, ctx, sim, n, nc, dt, world, newton_timed, p_timed):
    """The timed steps again, from the same initial state, through the
    public API with the state staged through page-locked host memory every
    step (host -> device before the step, device -> host after it).  The
    steps and Newton iterations are those of the timed pass."""
    from ressim_gb300 import api

    hp = api.PinnedArray(n)
    hN = api.PinnedArray(nc * n)
    hS = api.PinnedArray(3 * n)
    sim.restore_state()
    p, N, S = sim.state()
    hp.array[:] = p
    hN.array[:] = N.reshape(-1)
    e2e_newton = 0
    lib = api.lib()
    barrier(world)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.set_state(hp.array, hN.array)
        info = sim.step(dt)
        e2e_newton += info.newton_iterations
        ctx.check(lib.rsg_sim_get_state(sim.h, abi.dptr(hp.array), abi.dptr(hN.array), abi.dptr(hS.array)),
                  "get_state")
    ctx.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world)
    e2e_units = sum_over_ranks(float(n) * e2e_newton, world)
    h2d = (1 + nc) * n * 8
    d2h = (1 + nc + 3) * n * 8
    return {"value": e2e_units / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "newton_iterations": e2e_newton, "same_steps_as_timed": e2e_newton == newton_timed,
            "max_rel_pressure_diff_vs_timed": float(np.max(np.abs(hp.array - p_timed) / np.abs(p_timed)))}


def adjoint_leg(args, ctx, mesh, case, fluid, co, srcs, init, n, world):
    """Discrete adjoint on the same grid and physics: a recorded forward run
    of args.adj_steps steps from the initial state (Newton converged to a
    largest relative pressure change of 1e-8, so that the pressure equation
    holds at each step's end), checkpoints every args.adj_every steps,
    objective = oil moles produced into the producer column; then the
    backward sweep (recomputing every block but the last from its
    checkpoint) to dJ/dlog k of every cell.  Device time of both sweeps with
    CUDA events; the gradient's cost is backward / forward."""
    from ressim_gb300 import api

    spec = W.runspec(rtol=args.rtol, atol=1e-50, ptol=1e-8, stop_rule=1, max_newton=30)
    sim = api.Discretisation(ctx, mesh, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    dts = [case["dt"]] * args.adj_steps
    barrier(world)
    ctx.synchronize()
    ctx.timer_record(4)
    J, finfo = sim.forward(dts, args.adj_every, case["producer"], [0.0, 1.0])
    ctx.timer_record(5)
    grad, _, _, binfo = sim.backward(rtol=args.adj_rtol)
    ctx.timer_record(6)
    ctx.synchronize()
    fwd = max_over_ranks(ctx.timer_elapsed_ms(4, 5) / 1e3, world)
    bwd = max_over_ranks(ctx.timer_elapsed_ms(5, 6) / 1e3, world)
    return {"grid": f"{args.ni}x{args.nj}x{args.nk}", "parameters": n, "steps": args.adj_steps,
            "checkpoint_every": args.adj_every, "objective_oil_mol": J, "forward_s": fwd, "backward_s": bwd,
            "backward_over_forward": bwd / fwd, "newton_iterations": finfo.newton_iterations,
            "forward_linear_iterations": finfo.linear_iterations, "recomputed_steps": binfo.recomputed_steps,
            "adjoint_linear_iterations": binfo.adjoint_linear_iterations, "adjoint_rtol": args.adj_rtol,
            "grad_abs_max": float(np.max(np.abs(grad))), "grad_finite": bool(np.all(np.isfinite(grad)))}


def amg_leg(args, ctx, mesh, case, fluid, co, srcs, init, n, world):
    """MTJ's smoothed-aggregation AMG on the benchmark's first pressure
    system (the Jacobian and residual of the first Newton iteration): FP64
    GMRES(30) + AMG, and the mixed-precision solver (FP64 flexible GMRES
    around FP32 BiCGstab) with the FP32 AMG hierarchy, both to the
    benchmark's relative tolerance from x = 0.  Reported: setup wall time
    (aggregation, smoothed interpolation, Galerkin products and SSOR plans
    on the GPU, with their host-side planning), solve device time and
    iterations, the V-cycle's device time from the event-bracketed kernel
    families, its algorithmic bytes (level operators and interpolation read
    by the four SSOR sweeps, the residual, restriction and prolongation) and
    their fraction of the HBM peak, and the two solutions' difference.
    BiCGstab + AMG, the configuration's FP64 pairing, diverges on this
    system as it does in MTJ (the oracle's and the GPU's tests show it), so
    GMRES is the Krylov method here.  MTJ's left-preconditioned GMRES(30)
    with this AMG stalls on the 524,288-cell system (the preconditioned
    residual falls by about 10x in 300 iterations), so the FP64 run is
    capped at --amg-fp64-iters iterations and reports its per-iteration and
    per-V-cycle cost; the mixed solver converges and runs to the tolerance."""
    from ressim_gb300 import api

    spec = W.runspec(ptol=1e300, rtol=1e-2)
    sim = api.Discretisation(ctx, mesh, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    sim.enable_jacobian_capture()
    sim.step(case["dt"])
    rp, col = mesh.pattern(0)
    val, rhs = sim.jacobian(len(col))
    sim.release()
    A = api.CompRowMatrix(ctx, n, rp, col, val)
    hbm, peak_kind = peaks()
    out = {"system": f"first pressure Jacobian of the {args.ni}x{args.nj}x{args.nk} case", "rtol": args.rtol}
    vfam = ("amg_copy", "amg_zero", "amg_resid", "amg_restrict", "amg_prolong", "amg_direct", "amg_coarse_cvt",
            "ssor_fwd", "ssor_bwd", "ssor_copy", "ssor_fwd_f32", "ssor_bwd_f32")
    xs = {}
    for name, cls, cap in (("fp64_gmres", api.GMRES, args.amg_fp64_iters), ("mixed", api.MixedFGMRES, 200)):
        s = cls(ctx, abi.PC_AMG, rtol=args.rtol, atol=1e-50, max_iter=cap)
        ctx.synchronize()
        t0 = time.perf_counter()
        s.set_matrix(A)
        ctx.synchronize()
        setup_ms = (time.perf_counter() - t0) * 1e3
        levels = s.amg_levels()
        sizes = [s.amg_level_sizes(k) for k in range(levels)]
        ctx.set_profiling(True)
        ctx.profile_reset()
        ctx.timer_record(10)
        x = s.solve(A, rhs, np.zeros(n), raise_on_fail=False)
        ctx.timer_record(11)
        ctx.synchronize()
        prof = ctx.profile()
        ctx.set_profiling(False)
        solve_ms = ctx.timer_elapsed_ms(10, 11)
        cycles = prof.get("amg_direct", (0.0, 0))[1]
        vms = sum(prof[f][0] for f in vfam if f in prof)
        f32 = name == "mixed"
        eb, vb = (8, 4) if f32 else (12, 8)  # bytes per stored entry (value + index), per vector element
        vbytes = 0
        for k, (ln, lnnz, lc, pnnz) in enumerate(sizes):
            if k == levels - 1:
                break
            vbytes += 4 * (eb * lnnz + 4 * vb * ln)  # four SSOR sweeps: row entries, b, x, half iterate
            vbytes += eb * lnnz + 3 * vb * ln        # residual
            vbytes += 2 * (eb * pnnz + vb * (ln + lc))  # restriction and prolongation
        per_cycle = vms / cycles if cycles else None
        info = s.last_info
        out[name] = {"levels": levels, "level_rows": [int(z[0]) for z in sizes], "setup_ms": setup_ms,
                     "solve_ms": solve_ms, "iterations": info.iterations, "max_iterations": cap,
                     "status": abi.STATUS.get(info.reason), "ms_per_iteration": solve_ms / max(1, info.iterations),
                     "residual_reduction": info.residual / info.initial_residual if info.initial_residual else None,
                     "inner_iterations": info.inner_iterations if f32 else None, "v_cycles": cycles,
                     "v_cycle_ms": per_cycle, "v_cycle_bytes": vbytes,
                     "v_cycle_gbs": vbytes / (per_cycle / 1e3) / 1e9 if per_cycle else None,
                     "v_cycle_hbm_frac": (vbytes / (per_cycle / 1e3) / 1e9 / hbm) if per_cycle else None,
                     "peak_source": peak_kind}
        xs[name] = x
        s.release()
    out["true_rel_residual_mixed"] = float(np.linalg.norm(rhs - A.mult(xs["mixed"])) / np.linalg.norm(rhs)) \
        if hasattr(A, "mult") else None
    A.release()
    return out


def mixed_leg(args, ctx, mesh, case, fluid, co, srcs, init, fp64_sim, n, dt, fp64_s, p_fp64, world):
    """The same steps with the mixed-precision pressure solver (FP64 flexible
    GMRES around FP32 BiCGstab + FP32 ILU(0)) to the same relative residual:
    the first K steps from the initial state after W warm-up steps, exactly
    as the FP64 line times them, so the speed-up compares the same steps;
    the pressures after those steps against the FP64 line's; and the largest
    relative pressure difference after one more step taken by both from the
    same state."""
    from ressim_gb300 import api

    spec = W.runspec(method=abi.FGMRES_MIXED, rtol=args.rtol, atol=1e-50, inner_iterations=int(args.inner[0]),
                     inner_tolerance=args.inner[1])
    sim = api.Discretisation(ctx, mesh, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    sim.save_state()
    for _ in range(args.warmup):
        sim.step(dt)
    sim.restore_state()
    steps = args.mixed_steps if args.mixed_steps > 0 else args.steps
    barrier(world)
    ctx.synchronize()
    newton = linear = 0
    ctx.timer_record(2)
    for _ in range(steps):
        info = sim.step(dt)
        newton += info.newton_iterations
        linear += info.linear_iterations
    ctx.timer_record(3)
    ctx.synchronize()
    dev_s = max_over_ranks(ctx.timer_elapsed_ms(2, 3) / 1e3, world)
    units = sum_over_ranks(float(n) * newton, world)
    p, N, _ = sim.state()
    diff_k = float(np.max(np.abs(p - p_fp64) / np.abs(p_fp64))) if steps == args.steps else None
    sim.set_state(p, N)
    fp64_sim.set_state(p, N)
    # the comparison step is also the event-profiled one (per-kernel times)
    ctx.set_profiling(True)
    ctx.profile_reset()
    sim.step(dt)
    prof = ctx.profile()
    ctx.set_profiling(False)
    fp64_sim.step(dt)
    pm = sim.state()[0]
    pd = fp64_sim.state()[0]
    ms = dev_s * 1e3 / steps
    # FP32 SpMV of the inner solver: 4 B value + 4 B column per entry, row
    # length, x, y and the dot operand per row
    rp, col = mesh.pattern(0)
    f32_bytes = 8 * len(col) + 16 * n
    hbm, peak_kind = peaks()
    inner = None
    if "inner_spmv_dot" in prof:
        t_ms, cnt = prof["inner_spmv_dot"]
        gbs = f32_bytes / (t_ms / cnt / 1e3) / 1e9
        inner = {"kernel": "k_f32_spmv_dot", "launches": cnt, "avg_launch_us": round(t_ms / cnt * 1e3, 2),
                 "bytes_per_launch": f32_bytes, "achieved_gbs": round(gbs, 1), "peak": hbm,
                 "frac": round(gbs / hbm, 4), "peak_source": peak_kind}
    out = {"value": units / dev_s, "unit": METRIC, "ms_per_step": ms, "steps": steps,
           "newton_iterations": newton, "outer_iterations": linear,
           "inner": {"iterations": int(args.inner[0]), "rtol": args.inner[1]},
           "max_rel_pressure_diff_vs_fp64_after_steps": diff_k,
           "max_rel_pressure_diff_vs_fp64_one_step": float(np.max(np.abs(pm - pd) / np.abs(pd))),
           "inner_spmv": inner}
    if steps == args.steps:
        out["speedup_vs_fp64_same_steps"] = fp64_s / dev_s
    return out


def finish(args, ctx, mesh, sim, n, world, units, dev_s, wall, launches, clk, newton, linear, dt, e2e, rank=0):
    from ressim_gb300 import api

    # per-kernel device times from a separate profiled step (not the timed one)
    prof = {}
    if not args.no_kernel_profile:
        ctx.set_profiling(True)
        ctx.profile_reset()
        sim.step(dt)
        prof = ctx.profile()
        ctx.set_profiling(False)
    rp, col = mesh.pattern(0)
    lower_b, upper_b = sweep_bytes(rp, col)
    hbm, peak_kind = peaks()
    fam_bytes = {"ilu_lower": lower_b, "ilu_upper": upper_b}
    dominant = max(prof.items(), key=lambda kv: kv[1][0])[0] if prof else None
    sweeps = {k: v for k, v in prof.items() if k in fam_bytes}
    roof = None
    if sweeps:
        k = max(sweeps.items(), key=lambda kv: kv[1][0])[0]
        tot_ms, cnt = sweeps[k]
        per_launch = tot_ms / cnt / 1e3
        achieved = fam_bytes[k] / per_launch / 1e9
        traffic = NCU_TRAFFIC.get((args.ni, args.nj, args.nk), {}).get(k)
        roof = {"bound": "hbm", "kernel": k, "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 5), "traffic": traffic,
                "traffic_source": NCU_TRAFFIC_SOURCE if traffic else None, "peak_source": peak_kind,
                "bytes_per_launch": fam_bytes[k], "avg_launch_us": round(per_launch * 1e6, 2)}
    spmv_ms = prof.get("spmv_dot", (0, 1))
    spmv_bytes = 12 * len(col) + 4 * (n + 1) + 16 * n + 8 * n
    spmv = {"kernel": "k_spmv_dot",
            "achieved_gbs": round(spmv_bytes / (spmv_ms[0] / spmv_ms[1] / 1e3) / 1e9, 1) if spmv_ms[0] else None,
            "bytes_per_launch": spmv_bytes}
    if spmv["achieved_gbs"]:
        spmv.update(peak=hbm, frac=round(spmv["achieved_gbs"] / hbm, 4), peak_source=peak_kind,
                    avg_launch_us=round(spmv_ms[0] / spmv_ms[1] * 1e3, 2), launches=spmv_ms[1])
    total_ms = sum(v[0] for v in prof.values()) or 1.0
    shares = {k: round(v[0] / total_ms, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])[:8]}

    result = {
        "metric": METRIC,
        "value": units / dev_s,
        "unit": METRIC,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_s * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded lognormal permeability, perturbed grid, five-spot)",
        "config": config_of(args, len(col), dt),
        "newton_iterations": newton,
        "linear_iterations": linear,
        "l2": "matrix and factors (>300 MB) exceed the 129 MB L2",
        "parallelism": f"replicas x{world}",
        "e2e": e2e,
        "gpu_launches": launches,
        "sweep_mode": {-1: "undecided", 0: "one launch per level", 1: "one cluster walks all levels",
                       2: "one cluster, values pushed through distributed shared memory"}.get(
            api.lib().rsg_sweep_mode()),
        "roofline": roof,
        "spmv": spmv,
        "kernel_shares": shares,
        "dominant_kernel": dominant,
        "clocks": clk,
        "wall_s": wall,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args)
    return result


def ensemble_leg(args):
    """Ensemble of two-phase realisations (the batched-ensemble
    configuration): members with grids drawn uniformly between 32x32x8 and
    96x96x24 and their own seeded permeability.  Every arm times the same
    first time step from the initial state (each member is retracted after
    each step):
    * serial: the members stepped one after another, FP64 BiCGstab + ILU(0)
      (the plain FP64 GPU path, the configuration's reference point);
    * concurrent: rsg_ensemble_step, members on their own streams from host
      threads;
    * batched: rsg_ensemble_step_batched, all members' pressure solves in
      one persistent launch per Newton iteration, FP64 ILU(0) walks;
    * batched_mixed: the same launch with the mixed-precision solver (FP64
      flexible GMRES around 10 FP32 BiCGstab + FP32 ILU(0) steps), with its
      largest pressure difference against the serial FP64 step.
    Wall time around each call (host-driven Newton loop included).  The
    members stop Newton on max |dp/p| (RunSpec's alternative rule): the
    reference rule's signed pressure change of one cell sits at the linear
    solver's rounding level once converged, so its iteration count would
    follow the last bits of each arm's dot products."""
    from ressim_gb300 import api

    sizes = W.ensemble_sizes(args.ensemble)
    members = []
    try:
        for k, (ni, nj, nk) in enumerate(sizes):
            c = api.Context(0)
            sim, case = W.build_two_phase_sim(c, ni, nj, nk, seed=100 + k, rtol=args.rtol, stop_rule=1)
            members.append((c, sim, case, ni * nj * nk))
        sims = [m[1] for m in members]
        dts = [m[2]["dt"] for m in members]

        def retract_all():
            for m in members:
                m[1].retract()

        def timed(fn):
            fn()  # warm-up
            retract_all()
            t0 = time.perf_counter()
            infos = fn()
            t = time.perf_counter() - t0
            units = sum(m[3] * inf.newton_iterations for m, inf in zip(members, infos))
            return units / t, t, infos

        def serial():
            return [m[1].step(m[2]["dt"]) for m in members]

        def concurrent():
            infos, sts = api.ensemble_step(sims, dts)
            if sts.any():
                raise RuntimeError(f"ensemble member failed: {sts.tolist()}")
            return infos

        def batched(precision):
            def f():
                infos, sts = api.ensemble_step_batched(sims, dts, precision=precision)
                if sts.any():
                    raise RuntimeError(f"batched ensemble member failed: {sts.tolist()}")
                return infos
            return f

        v_ser, t_ser, _ = timed(serial)
        p_ser = [m[1].state()[0].copy() for m in members]
        retract_all()
        v_conc, t_conc, _ = timed(concurrent)
        retract_all()
        v_bat, t_bat, inf_bat = timed(batched(0))
        d64 = max(float(np.max(np.abs(m[1].state()[0] - p) / np.abs(p))) for m, p in zip(members, p_ser))
        retract_all()
        v_mix, t_mix, inf_mix = timed(batched(1))
        dmix = max(float(np.max(np.abs(m[1].state()[0] - p) / np.abs(p))) for m, p in zip(members, p_ser))
        retract_all()
    finally:
        for m in members:
            m[0].close()
    return {"members": len(sizes), "cells": int(sum(m[3] for m in members)),
            "grids": "each axis uniform in 32..96 x 32..96 x 8..24 (seeded)",
            "step": "the first time step from the initial state, Newton converged", "unit": METRIC,
            "serial_value": v_ser, "concurrent_value": v_conc, "batched_value": v_bat,
            "batched_mixed_value": v_mix,
            "value": v_mix, "speedup_vs_serial": v_mix / v_ser,
            "speedup_batched_fp64_vs_serial": v_bat / v_ser, "speedup_concurrent_vs_serial": v_conc / v_ser,
            "seconds": {"serial": t_ser, "concurrent": t_conc, "batched": t_bat, "batched_mixed": t_mix},
            "newton_iterations": {"batched": int(sum(i.newton_iterations for i in inf_bat)),
                                  "batched_mixed": int(sum(i.newton_iterations for i in inf_mix))},
            "max_rel_pressure_diff_vs_serial_fp64": {"batched": d64, "batched_mixed": dmix}}


def flash_leg(args):
    """Per-cell Peng-Robinson phase state with isothermal flash
    (CubicEquationOfState.calculatePhaseState) on the compositional
    configuration's size, 256x256x16 = 1,048,576 cells: water plus three
    seeded hydrocarbon pseudo-components, seeded p in 60-400 bar, T in
    300-400 K.  Timed through the C ABI with host arrays (copies included):
    a cold call (Wilson K-values) and a warm call from the returned phases.
    The oracle (single thread) times the same cold call."""
    from oracle import oracle as O
    from ressim_gb300 import api

    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    n = args.flash_cells
    p, T, N = W.compositional_cells(n, f.nc)
    ctx = api.Context(0)
    try:
        api.cubic_phase_state(ctx, f, p[:1024], T[:1024], N[:, :1024], per_cell=True)  # first-launch costs
        t0 = time.perf_counter()
        ph, its, sts = api.cubic_phase_state(ctx, f, p, T, N, per_cell=True)
        t_cold = time.perf_counter() - t0
        t0 = time.perf_counter()
        ph2, its2, sts2 = api.cubic_phase_state(ctx, f, p, T, N, ph, per_cell=True)
        t_warm = time.perf_counter() - t0
    finally:
        ctx.close()
    out = {"cells": n, "unit": "cells/s", "cold_value": n / t_cold, "warm_value": n / t_warm,
           "mean_flash_iterations_cold": float(its.mean()), "mean_flash_iterations_warm": float(its2.mean()),
           "two_phase_cells": int(((ph[1, 0] > 0) & (ph[2, 0] > 0)).sum()),
           "failed_cells": int((sts != 0).sum())}
    if not args.no_cpu_baseline:
        t0 = time.perf_counter()
        try:
            O.cubic_phase_state(f, p, T, N)
            out["cpu_oracle_cold_value"] = n / (time.perf_counter() - t0)
        except O.OracleError as e:
            out["cpu_oracle_error"] = str(e)
        out["cpu_cores"] = 1
    return out


def compositional_leg(args):
    """Compositional steps end to end (Peng-Robinson flash in every cell's
    property evaluation, FP64 BiCGstab + ILU(0) pressure solve, explicit
    molar update) on a line drive of the compositional fluid, 64x64x16 by
    default, dt = 2000 s with negative moles truncated; against the oracle
    on the same grid and steps."""
    from oracle import oracle as O
    from ressim_gb300 import api

    ni, nj, nk = args.comp_grid
    keep = abi.Keep()
    f = W.compositional_fluid(keep)
    case = W.compositional_case(ni, nj, nk, dt=2000.0)
    srcs = W.build_compositional_sources(keep, case, f.nc)
    init = W.build_compositional_initial(case, f.nc)
    spec = W.runspec(rtol=args.rtol)
    spec.truncate_negative_moles = 1  # RunSpec TruncateNegativeMoles: the explicit update overshoots in a few cells
    ctx = api.Context(0)
    try:
        mesh = api.Mesh(ctx, 3, ni, nj, nk, case["perm"], coords=case["nodes"])
        mesh.compute_mpfa()
        sim = api.Discretisation(ctx, mesh, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
        sim.step(case["dt"])  # warm-up
        ctx.synchronize()
        newton = 0
        t0 = time.perf_counter()
        for _ in range(args.comp_steps):
            newton += sim.step(case["dt"]).newton_iterations
        ctx.synchronize()
        secs = time.perf_counter() - t0
        # the same steps with the mixed-precision pressure solver (FP64 flash
        # and Rachford-Rice, FP32 inner Krylov stage)
        mspec = W.runspec(rtol=args.rtol, method=abi.FGMRES_MIXED, inner_iterations=int(args.inner[0]),
                          inner_tolerance=args.inner[1])
        mspec.truncate_negative_moles = 1
        msim = api.Discretisation(ctx, mesh, f, W.corey(), case["porosity"], case["compaction"], srcs, init, mspec)
        msim.step(case["dt"])  # warm-up
        ctx.synchronize()
        mnewton = 0
        t0 = time.perf_counter()
        for _ in range(args.comp_steps):
            mnewton += msim.step(case["dt"]).newton_iterations
        ctx.synchronize()
        msecs = time.perf_counter() - t0
        pm, pd = msim.state()[0], sim.state()[0]
    finally:
        ctx.close()
    n = ni * nj * nk
    out = {"grid": f"{ni}x{nj}x{nk}", "components": f.nc, "steps": args.comp_steps, "newton_iterations": newton,
           "dt_s": case["dt"],
           "value": n * newton / secs, "unit": METRIC, "mixed_value": n * mnewton / msecs,
           "mixed_max_rel_pressure_diff_vs_fp64": float(np.max(np.abs(pm - pd) / np.abs(pd)))}
    if not args.no_cpu_baseline:
        om = O.Mesh(3, ni, nj, nk, coords=case["nodes"], perm=case["perm"])
        om.mpfa()
        osim = O.Simulator(om, f, W.corey(), case["porosity"], case["compaction"], srcs, init, spec)
        osim.step(case["dt"])
        on = 0
        t0 = time.perf_counter()
        for _ in range(args.comp_steps):
            on += osim.step(case["dt"]).newton_iterations
        out["cpu_oracle_value"] = n * on / (time.perf_counter() - t0)
        out["cpu_cores"] = 1
    return out


def oracle_full(args, one_newton=False):
    """The oracle (single-threaded C++ restatement of RS + MTJ) on the full
    workload from its initial state.  With one_newton the pressure tolerance
    is 1e300, so that a step is one Newton iteration: assembly, BiCGstab +
    ILU(0) to the same relative residual and the explicit molar-mass update
    over every cell (the bounded CPU-baseline sample)."""
    from oracle import oracle as O

    case, keep, fluid, co, srcs, init, spec = build_case(args)
    if one_newton:
        spec.pressure_tolerance = 1e300
    m = O.Mesh(3, args.ni, args.nj, args.nk, coords=case["nodes"], perm=case["perm"])
    m.mpfa()
    sim = O.Simulator(m, fluid, co, case["porosity"], case["compaction"], srcs, init, spec)
    return sim, case, keep, m


def oracle_steps(sim, case, steps):
    newton = linear = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        info = sim.step(case["dt"])
        newton += info.newton_iterations
        linear += info.linear_iterations
    return newton, linear, time.perf_counter() - t0


def cpu_baseline(args):
    sim, case, keep, m = oracle_full(args, one_newton=True)
    newton, linear, secs = oracle_steps(sim, case, args.cpu_steps)
    n = args.ni * args.nj * args.nk
    return {"value": n * newton / secs, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"oracle (C++ restatement of RS+MTJ, single thread, as the reference's solvers are) on the "
                      f"full {args.ni}x{args.nj}x{args.nk} case: the first {args.cpu_steps} time step(s) from the "
                      f"initial state, one Newton iteration each, {linear} BiCGstab iterations, {secs:.1f} s"}


def java_probe():
    """RS and MTJ are Java; the reference itself runs only where a JVM is."""
    java = shutil.which("java")
    return {"java": java, "reference_jvm": "unavailable on this box (no JVM)" if java is None else
            "present, but the timed reference is the C++ port of the same Java code"}


def run_reference(args):
    """The same K steps from the initial state on the oracle, with the same
    converged Newton loop as the GPU line.  Warm-up: W steps of a 16x16x4
    case of the same physics (the CPU code has no device state or first-launch
    cost to warm; running W full steps would only add W x ~45 s)."""
    small = argparse.Namespace(**vars(args))
    small.ni, small.nj, small.nk = 16, 16, 4
    wsim, wcase, _, _ = oracle_full(small)
    oracle_steps(wsim, wcase, args.warmup)
    del wsim
    sim, case, keep, m = oracle_full(args)
    rp, col = m.pattern(0)
    newton, linear, secs = oracle_steps(sim, case, args.steps)
    n = args.ni * args.nj * args.nk
    value = n * newton / secs
    return {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": METRIC,
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded lognormal permeability, perturbed grid, five-spot)",
        "config": config_of(args, len(col), case["dt"]),
        "newton_iterations": newton,
        "linear_iterations": linear,
        "jvm": java_probe(),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": 1, "kind": "port",
                         "sample": f"the first {args.steps} time steps from the initial state on the full case, "
                                   f"Newton converged as on the GPU ({newton} Newton and {linear} BiCGstab "
                                   f"iterations, {secs:.1f} s); warm-up: {args.warmup} steps of a 16x16x4 case"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


_dist = None


def init_dist(world):
    global _dist
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        _dist = dist


def barrier(world):
    if _dist:
        _dist.barrier()


def max_over_ranks(v, world):
    if not _dist:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    _dist.all_reduce(t, op=_dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, world):
    if not _dist:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    _dist.all_reduce(t, op=_dist.ReduceOp.SUM)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="resgpu", choices=["resgpu", "reference"])
    ap.add_argument("--ni", type=int, default=128)
    ap.add_argument("--nj", type=int, default=128)
    ap.add_argument("--nk", type=int, default=32)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end pass (profiling runs)")
    ap.add_argument("--no-kernel-profile", action="store_true", help="skip the event-bracketed per-kernel pass")
    ap.add_argument("--mixed-steps", type=int, default=0,
                    help="steps timed with the mixed-precision pressure solver (0: the same K steps as the FP64 "
                         "line, -1: skip)")
    ap.add_argument("--amg", type=int, default=1, help="AMG leg on the first pressure system (0: skip)")
    ap.add_argument("--amg-fp64-iters", type=int, default=30, help="AMG leg: iteration cap of FP64 GMRES + AMG")
    ap.add_argument("--ensemble", type=int, default=64, help="ensemble members (0: skip)")
    ap.add_argument("--flash-cells", type=int, default=1048576,
                    help="cells of the Peng-Robinson flash leg (0: skip)")
    ap.add_argument("--comp-steps", type=int, default=1, help="timed steps of the compositional leg (0: skip)")
    ap.add_argument("--comp-grid", type=int, nargs=3, default=[64, 64, 16])
    ap.add_argument("--adj-steps", type=int, default=50, help="steps of the adjoint leg (0: skip)")
    ap.add_argument("--adj-every", type=int, default=10, help="adjoint leg: steps per checkpoint")
    ap.add_argument("--adj-rtol", type=float, default=1e-8, help="adjoint leg: transposed-solve tolerance")
    ap.add_argument("--inner", type=float, nargs=2, default=[10, 1e-3],
                    help="mixed solver: FP32 inner iterations and inner relative tolerance")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return
    init_dist(world)
    res = run_resgpu(args, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
