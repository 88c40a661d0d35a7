#!/usr/bin/env python3
"""Throughput of the LDDRK time step (rk.f90:12-75) on GB300.

Workload: the 4096x2048 Navier-Stokes case on the y-stretched grid (FP64,
rho,u,v,p), one "step" = one call of rk_euler over the whole grid (six
stages: RHS, update, buffer, both filters, boundary conditions).  Metric:
Mpt-steps/s = imax*jmax*steps / s / 1e6.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank advances its own replica on its own GPU (the path
has no exchange step: replicas only); the line reports the whole-job rate
over the slowest rank.  `--impl reference` times the CPU oracle (the C
restatement of the Fortran reference, which cannot be compiled here) on the
host cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpt-steps/s, FP64 vs split-precision at stated p' error; adjoint/fwd cost"
UNIT = "Mpt-steps/s"

# Algorithmic HBM bytes per grid point of one launch of each kernel class
# (every input read once, every output written once; nk = 4, Navier-Stokes):
#   k_prim:     rho, p in; T, 1/rho out                          4*8
#   k_first:    U(4) + T in; dU/dx(4), dU/dy(4), tau(3), k*grad T(2) out
#   k_update:   U, w, dU/dx, dU/dy, tau, k*grad T, 1/rho in; U, w out
#   k_filter_*: U in, U out
BYTES_PER_POINT = {"k_prim": 32, "k_first": 144, "k_update": 240, "k_filter_x": 64,
                   "k_filter_y": 64, "k_bc": 0, "k_stage_sin": 0}
# FP64 work per grid point of one launch, from ncu's executed-instruction
# counts of each kernel on a 2048x2048 Navier-Stokes grid (nk = 4): flops (2
# per DFMA, 1 per DADD/DMUL) and FP64-pipe thread instructions (DFMA, DADD,
# DMUL and the FP32<->FP64 conversions, which share that pipe on GB300).
FP64_FLOP_PER_POINT = {"k_prim": 12.0, "k_first": 113.15, "k_update": 111.43,
                       "k_filter_x": 82.44, "k_filter_y": 82.44}
FP64_INST_PER_POINT = {"k_prim": 7.0, "k_first": 81.03, "k_update": 71.84,
                       "k_filter_x": 53.78, "k_filter_y": 53.78}
# DRAM bytes (read + write) per point of one launch from the same capture
# (2048x2048), scaled to a launch by the number of points.
TRAFFIC_PER_POINT = {"k_prim": 21.3, "k_first": 129.9, "k_update": 230.5,
                     "k_filter_x": 56.6, "k_filter_y": 56.0}
# DFMA throughput of a register-only loop measured on a GB300 (1.68 DFMA per
# clock per SM at 2.07 GHz), used when ns_fp64_peak() cannot run
FP64_PEAK_FALLBACK_TFLOPS = 1.19
# FP64-pipe thread instructions per point-step of the whole step (sum of the
# per-launch counts above over the step's 36 launches, nk = 4)
FP64_INST_PER_POINT_STEP = 1605
STEP_BYTES_FUSED_MIN = 1536  # compulsory bytes per point-step of a fused FP64 design, nk = 4


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region (200 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_case(args):
    from navierstokes_gb300 import cases
    return cases.stretched_ns_case(imax=args.imax, jmax=args.jmax, nk=args.nk)


def workload_config(case, extra=None):
    cfg = {"workload": f"Navier-Stokes {case.imax}x{case.jmax}, y stretched toward the "
                       "centreline (eta = tanh(2.5y)/tanh(2.5)), M=0.5, Re=1000, Pr=0.72, "
                       "pulse 1e-3 + isentropic vortex 0.1, D=40, sigma_f=0.2, "
                       f"dt = min(CFL 0.5, viscous limit) = {case.dt:.4g}",
           "imax": case.imax, "jmax": case.jmax, "nk": case.nk, "precision": "fp64",
           "l2": "inputs larger than L2 (state and work arrays ~2 GB)",
           "parallelism": "replicas only (one independent grid per GPU)"}
    if extra:
        cfg.update(extra)
    return cfg


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            import torch
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    return world, rank, local, pg


def max_over_ranks(pg, x, device="cpu"):
    """The largest x over all ranks: the slowest replica's time."""
    if pg is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, points, steps, seconds):
    """Mpt-steps/s of the whole job: every replica's points over the slowest."""
    return world * points * steps / seconds / 1e6


def run_reference(args, world, rank):
    """CPU oracle on all host threads; rank 0 only."""
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    case = build_case(args)
    config = workload_config(case)
    # one step of the full grid first, to size the sample
    o = oracle.Oracle(case)
    U = case.U0.copy()
    t0 = time.perf_counter()
    o.run(U, 0, 1)
    t_full = time.perf_counter() - t0
    budget = 150.0
    jmax_s = case.jmax
    if (args.steps + args.warmup) * t_full > budget:
        frac = budget / ((args.steps + args.warmup) * t_full)
        jmax_s = max(64, int(case.jmax * frac) // 16 * 16)
    if jmax_s != case.jmax:
        from navierstokes_gb300 import cases
        o.close()
        case = cases.stretched_ns_case(imax=case.imax, jmax=jmax_s, nk=case.nk)
        o = oracle.Oracle(case)
        U = case.U0.copy()
    for it in range(args.warmup):
        o.run(U, it, 1)
    t0 = time.perf_counter()
    for it in range(args.steps):
        o.run(U, args.warmup + it, 1)
    dt = time.perf_counter() - t0
    val = case.points * args.steps / dt / 1e6
    sample = (f"{args.steps} timed steps of a {case.imax}x{case.jmax} grid "
              f"({'full grid' if jmax_s == args.jmax else f'rows cropped from {args.jmax} to bound the run; the rate is per point-step'}), "
              f"{threads} OpenMP threads")
    line = {"metric": METRIC, "value": val, "unit": UNIT, "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: analytic pulse + isentropic vortex on the stretched grid",
            "config": config,
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Algorithmic HBM bytes per point of one launch of the split-precision
# kernels, averaged over the six stages: q' is 7 FP32 planes (rho'; u', v',
# p' hi; their lo parts) = 28 B; the stage reads q' and w (4 x FP64) and
# writes both, except that stage 0 does not read w and stage 5 does not
# write it (28 + 32 + 28 + 32 = 120 B, minus 32 B in two of six launches);
# each filter reads and writes q'.
SPLIT_BYTES_PER_POINT = {"k_split_stage": (6 * 120 - 2 * 32) / 6, "k_split_filter_x": 56,
                         "k_split_filter_y": 56}
SPLIT_STEP_BYTES_MIN = 6 * 120 - 2 * 32 + 12 * 56   # 1328 per point-step
# Navier-Stokes in split precision, per point-step: the stage kernel also
# reads the five FP32 viscous planes (20 B) and k_split_visc reads q' (28 B)
# and writes them (20 B) in every stage.
SPLIT_NS_STEP_BYTES_MIN = SPLIT_STEP_BYTES_MIN + 6 * (20 + 28 + 20)   # 1736
# NS_PREC_SPLIT32: q' is 4 FP32 planes (16 B)
SPLIT32_BYTES_PER_POINT = {"k_split_stage": (6 * 96 - 2 * 32) / 6, "k_split_filter_x": 32,
                           "k_split_filter_y": 32}


def split_study(args, local, hbm_peak):
    """The split-precision workload: Euler, 4096x4096 uniform grid, M = 0.5, pulse 1e-4,
    vortex 1e-3, 1000 steps; split precision (u', v', p' as FP32 pairs) and
    the all-FP32 split against plain FP64 (throughput of each and p' = p - p_b
    error at steps 100/500/1000)."""
    import ctypes as C
    import torch
    from navierstokes_gb300 import Solver, cases
    from navierstokes_gb300 import _lib as L
    case = cases.uniform_flow_case(imax=args.split_n, jmax=args.split_n)
    out = {"workload": f"Euler {case.imax}x{case.jmax} uniform grid, M=0.5, pulse 1e-4, "
                       f"isentropic vortex 1e-3, D=30, sigma_f=0.2, CFL 0.5, dt={case.dt:.3g}",
           "error_steps": args.split_error_steps}
    stream = torch.cuda.Stream()
    rates = {}
    states = {}
    kernels = {}
    for name, prec in (("fp64", L.NS_PREC_FP64), ("split", L.NS_PREC_SPLIT),
                       ("split32", L.NS_PREC_SPLIT32)):
        s = Solver(case, device=local, precision=prec)
        s.set_stream(stream.cuda_stream)
        s.set_state(case.U0)
        done = 0
        snaps = {}
        for n in args.split_error_steps:
            s.step(done, n - done)
            done = n
            snaps[n] = s.get_state()
        states[name] = snaps
        for it in range(args.warmup):
            s.step(done + it, 1)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            s.step(done + args.warmup + k, 1)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        rates[name] = {"value": case.points / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                       "gpu_launches_per_step": s.launches_per_step()}
        if name in ("split", "split32"):
            kernels = {} if name == "split" else kernels
            kms = (C.c_double * L.NS_KC_COUNT)()
            kn = (C.c_int * L.NS_KC_COUNT)()
            L.check(s.lib.ns_time_kernels(s._ctx, 20_000, 2, kms, kn), s._ctx)
            for k in range(L.NS_KC_COUNT):
                if kn[k]:
                    kname = s.lib.ns_kernel_name(k).decode()
                    bpp = (SPLIT_BYTES_PER_POINT if name == "split"
                           else SPLIT32_BYTES_PER_POINT).get(kname)
                    entry = {"ms_per_launch": kms[k], "launches_per_step": kn[k]}
                    if bpp:
                        gbs = bpp * case.points / (kms[k] * 1e-3) / 1e9
                        entry["achieved_gbs"] = gbs
                        entry["hbm_frac"] = gbs / hbm_peak
                    if name == "split":
                        kernels[kname] = entry
                    else:
                        rates[name].setdefault("kernels", {})[kname] = entry
        s.close()
    tot = sum(v["ms_per_launch"] * v["launches_per_step"] for v in kernels.values())
    for v in kernels.values():
        v["share"] = v["ms_per_launch"] * v["launches_per_step"] / tot
    dom = max(kernels, key=lambda n: kernels[n]["share"])
    def p_errors(mode):
        errs = {}
        for n in args.split_error_steps:
            a, b = states["fp64"][n], states[mode][n]
            dp = b[..., 3] - a[..., 3]
            pr = a[..., 3] - case.Ub[..., 3]
            errs[str(n)] = {"p_rel_l2": float(np.linalg.norm(dp) / np.linalg.norm(pr)),
                            "p_rel_max": float(np.max(np.abs(dp)) / np.max(np.abs(pr))),
                            "p_abs_max": float(np.max(np.abs(dp)))}
        return errs
    errs = p_errors("split")
    step_gbs = SPLIT_STEP_BYTES_MIN * case.points / (rates["split"]["ms_per_step"] * 1e-3) / 1e9
    out.update({"value": rates["split"]["value"], "unit": UNIT,
                "fp64_value": rates["fp64"]["value"],
                "speedup_vs_fp64": rates["split"]["value"] / rates["fp64"]["value"],
                "ms_per_step": rates["split"]["ms_per_step"],
                "fp64_ms_per_step": rates["fp64"]["ms_per_step"],
                "p_error_vs_fp64": errs,
                "roofline": {"bound": "hbm", "kernel": dom,
                             "achieved": kernels[dom].get("achieved_gbs"),
                             "peak": hbm_peak, "unit": "GB/s",
                             "frac": kernels[dom].get("hbm_frac"),
                             "step_bytes_per_point": SPLIT_STEP_BYTES_MIN,
                             "step_frac": step_gbs / hbm_peak},
                "kernels": kernels,
                "split32": {"what": "every perturbation one FP32 number (NS_PREC_SPLIT32)",
                            "value": rates["split32"]["value"], "unit": UNIT,
                            "ms_per_step": rates["split32"]["ms_per_step"],
                            "speedup_vs_fp64": rates["split32"]["value"] / rates["fp64"]["value"],
                            "p_error_vs_fp64": p_errors("split32"),
                            "kernels": rates["split32"].get("kernels")}})
    return out


def split_ns_study(args, local, hbm_peak):
    """The Navier-Stokes workload (4096x2048, y-stretched, M = 0.5, Re = 1000,
    pulse 1e-3 and vortex 0.1) in split precision against plain FP64: both
    run its 200 steps from the same start; throughput of each and the p'
    error at the end."""
    import torch
    from navierstokes_gb300 import Solver, cases
    from navierstokes_gb300 import _lib as L
    case = build_case(args)
    nsteps = args.split_ns_steps
    stream = torch.cuda.Stream()
    out = {"workload": f"Navier-Stokes {case.imax}x{case.jmax} (the main line's flow), "
                       f"{nsteps} steps", "unit": UNIT}
    finals = {}
    for name, prec in (("fp64", L.NS_PREC_FP64), ("split", L.NS_PREC_SPLIT)):
        with Solver(case, device=local, precision=prec) as s:
            s.set_stream(stream.cuda_stream)
            s.set_state(case.U0)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(0, nsteps)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / nsteps
            finals[name] = s.get_state()
            out[name] = {"value": case.points / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                         "launches_per_step": s.launches_per_step()}
    dp = finals["split"][..., 3] - finals["fp64"][..., 3]
    pr = finals["fp64"][..., 3] - case.Ub[..., 3]
    out["value"] = out["split"]["value"]
    gbs = SPLIT_NS_STEP_BYTES_MIN * case.points / (out["split"]["ms_per_step"] * 1e-3) / 1e9
    out["hbm"] = {"step_bytes_per_point": SPLIT_NS_STEP_BYTES_MIN, "achieved": gbs,
                  "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak}
    out["speedup_vs_fp64"] = out["split"]["value"] / out["fp64"]["value"]
    out["p_error_vs_fp64"] = {"p_rel_l2": float(np.linalg.norm(dp) / np.linalg.norm(pr)),
                              "p_rel_max": float(np.max(np.abs(dp)) / np.max(np.abs(pr))),
                              "at_step": nsteps}
    return out


def small_grid_study(local, steps=500):
    """The 201x201 Euler acoustic pulse, 500 steps from rest: the
    L2-resident, latency-bound case.  Device-resident FP64 steps timed with
    CUDA events, two ways: the step graph of ns_step (nk = 5, psi carried as
    the reference does, with the per-kernel times of one step), and one
    persistent cooperative launch per step (ns_batch with this one instance,
    nk = 4: psi is passive and the Euler case does not need it)."""
    import ctypes as C
    import torch
    from navierstokes_gb300 import Batch, Solver, cases
    from navierstokes_gb300 import _lib as L
    c = cases.acoustic_pulse_case()
    out = {"workload": f"Euler {c.imax}x{c.jmax} acoustic pulse, FP64, {steps} steps",
           "steps": steps, "unit": UNIT}
    stream = torch.cuda.Stream()
    with Solver(c, device=local) as s:
        s.set_stream(stream.cuda_stream)
        s.set_state(c.U0)
        s.step(0, 20)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.step(20, steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        kms = (C.c_double * L.NS_KC_COUNT)()
        kn = (C.c_int * L.NS_KC_COUNT)()
        L.check(s.lib.ns_time_kernels(s._ctx, 1000, 5, kms, kn), s._ctx)
        kernels = {s.lib.ns_kernel_name(k).decode(): {"ms_per_launch": kms[k],
                                                       "launches_per_step": kn[k]}
                   for k in range(L.NS_KC_COUNT) if kn[k]}
        launches = s.launches_per_step()
    out["graph"] = {"nk": c.nk, "value": c.points / (ms * 1e-3) / 1e6, "ms_per_step": ms,
                    "launches_per_step": launches, "kernels": kernels}
    c4 = cases.acoustic_pulse_case(nk=4)
    with Batch([c4], device=local, precision=L.NS_PREC_FP64) as b:
        b.set_stream(stream.cuda_stream)
        b.set_initial()
        ty, bps, _ = b.autotune(0, 5)
        b.set_initial()
        b.step(0, 20)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(20, steps)
        e1.record(stream)
        b.synchronize()
        torch.cuda.synchronize()
        msb = e0.elapsed_time(e1) / steps
        out["persistent"] = {"nk": 4, "value": c4.points / (msb * 1e-3) / 1e6,
                             "ms_per_step": msb, "tile_rows": ty, "blocks_per_sm": bps,
                             "launch": b.info()}
    out["value"] = max(out["graph"]["value"], out["persistent"]["value"])
    return out


def batch_study(args, local):
    """The parameter-sweep workload: 64 independent Euler instances, sizes log-uniform in
    [128, 1024] (multiples of 32), monopole sources, mean flow M ~ U[0, 0.6],
    numpy.random.default_rng(0); 300 steps in one persistent launch per step,
    FP64 and split precision, tiles autotuned."""
    import torch
    from navierstokes_gb300 import Batch, cases
    from navierstokes_gb300 import _lib as L
    cs = cases.sweep_cases(n=args.batch_n, seed=0)
    pts = sum(c.points for c in cs)
    out = {"workload": f"{len(cs)} Euler instances, Nx,Ny in [128,1024] log-uniform (seed 0), "
                       f"{pts} points in total, monopole sources, M ~ U[0,0.6], "
                       f"{args.batch_steps} steps", "points": pts}
    finals = {}
    for name, prec in (("fp64", L.NS_PREC_FP64), ("split", L.NS_PREC_SPLIT32)):
        b = Batch(cs, device=local, precision=prec)
        stream = torch.cuda.Stream()
        b.set_stream(stream.cuda_stream)
        b.set_initial()
        ty, bps, tms = b.autotune(0, 3)
        b.set_initial()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.step(0, args.batch_steps)
        e1.record(stream)
        b.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.batch_steps
        finals[name] = [b.get_state(q) for q in range(len(cs))]
        out[name] = {"value": pts / (ms * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": ms,
                     "tile_rows": ty, "blocks_per_sm": bps, "launch": b.info(),
                     "phase_ms_per_step": b.phase_times(args.batch_steps)}
        b.close()
    l2n = l2d = 0.0
    mx = mref = 0.0
    for q, c in enumerate(cs):
        dp = finals["split"][q][..., 3] - finals["fp64"][q][..., 3]
        pr = finals["fp64"][q][..., 3] - c.Ub[..., 3]
        l2n += float(np.sum(dp * dp))
        l2d += float(np.sum(pr * pr))
        mx = max(mx, float(np.max(np.abs(dp))))
        mref = max(mref, float(np.max(np.abs(pr))))
    out["split_speedup_vs_fp64"] = out["split"]["value"] / out["fp64"]["value"]
    out["split_p_error_vs_fp64"] = {"p_rel_l2": (l2n / l2d) ** 0.5, "p_rel_max": mx / mref,
                                    "at_step": args.batch_steps}
    return out


def adjoint_study(args, local):
    """The adjoint workload: Euler on 512x512 with M = 0.3, a Gaussian monopole
    source field (b = 32 cells) whose amplitude is the Keys-cubic
    interpolant of 16x16 controls ~ N(0, 1e-3) (seed 0), omega = 0.5, 2000
    steps; loss = sum over steps of p'^2 at 32 observers on a circle of
    radius 150 cells.  Times the plain FP64 forward (ns_step), the forward
    with the loss (every stage input kept when it fits, --adjoint-k 0; else
    checkpoints) and the reverse pass (stage derivatives or segments
    recomputed, then the stage adjoints; with checkpoints the recompute of
    one segment runs beside the reverse of the next), and checks the control
    gradient at two controls against central differences h = 1e-7."""
    import time
    from navierstokes_gb300 import Solver
    from navierstokes_gb300.adjoint import Adjoint, SourceProblem
    pb = SourceProblem(steps=args.adjoint_steps)
    c = pb.case
    out = {"workload": f"Euler {c.imax}x{c.jmax}, M=0.3, monopole field from 16x16 controls, "
                       f"omega=0.5, {pb.steps} steps, 32 observers at r=150",
           "steps": pb.steps, "checkpoint_every": args.adjoint_k}
    with Solver(c, device=local) as s:
        s.set_state(c.U0)
        s.step(0, 20)
        s.synchronize()
        s.set_state(c.U0)
        t0 = time.perf_counter()
        s.step(0, pb.steps)
        s.synchronize()
        t_plain = time.perf_counter() - t0
    with Adjoint(pb, checkpoint_every=args.adjoint_k, device=local) as adj:
        adj.set_field(pb.field(pb.controls))
        adj.forward(20)
        adj.backward()
        t0 = time.perf_counter()
        loss = adj.forward()
        t_fwd = time.perf_counter() - t0
        stored = adj.stored_bytes()
        t0 = time.perf_counter()
        gfield = adj.backward()
        t_bwd = time.perf_counter() - t0
        gc = pb.controls_grad(gfield)
        fd = []
        h = 1e-7
        for (a, b) in [(7, 8), (8, 7)]:
            cp = pb.controls.copy()
            cp[a, b] += h
            adj.set_field(pb.field(cp))
            lp = adj.forward()
            cp[a, b] -= 2 * h
            adj.set_field(pb.field(cp))
            lm = adj.forward()
            d = (lp - lm) / (2 * h)
            fd.append({"control": [a, b], "adjoint": gc[a, b], "fd": d,
                       "rel_err": abs(d - gc[a, b]) / abs(gc[a, b])})
    out.update({"loss": loss, "plain_forward_s": t_plain, "forward_with_loss_s": t_fwd,
                "backward_s": t_bwd, "backward_over_plain_forward": t_bwd / t_plain,
                "gradient_cost_over_plain_forward": (t_fwd + t_bwd) / t_plain,
                "plain_forward_value": c.points * pb.steps / t_plain / 1e6, "unit": UNIT,
                "fd_check": fd, "grad_norm": float(np.linalg.norm(gc)),
                "forward_storage": (f"every stage input kept: {stored / 1e9:.1f} GB" if stored
                                    else f"checkpoints every {args.adjoint_k or 100} steps")})
    return out


def cpu_baseline_sample(case, seconds=20.0):
    """Oracle on the host cores, a bounded sample of the same workload."""
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    o = oracle.Oracle(case)
    U = case.U0.copy()
    t0 = time.perf_counter()
    o.run(U, 0, 1)
    t1 = time.perf_counter() - t0
    n = max(1, min(8, int(seconds / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.run(U, 1, n)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": case.points * n / dt / 1e6, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{n} step(s) of the full {case.imax}x{case.jmax} grid after one "
                      f"untimed step, C oracle (-O3, OpenMP over lines)"}


def cpu_workloads_study(seconds=8.0):
    """The C oracle on every workload of this benchmark, on all host cores
    and on one core: a bounded sample of steps each (the per-step rate is
    what is reported).  The sweep times its 64 instances one after the
    other; the source problem times its forward step."""
    import oracle
    from navierstokes_gb300 import cases
    from navierstokes_gb300.adjoint import SourceProblem
    oracle.build()
    allc = os.cpu_count() or 1
    work = [("201x201 Euler pulse", [cases.acoustic_pulse_case()]),
            ("4096x2048 Navier-Stokes", [cases.stretched_ns_case()]),
            ("4096x4096 Euler, pulse + vortex", [cases.uniform_flow_case()]),
            ("64 Euler instances (seed 0)", cases.sweep_cases(n=64, seed=0)),
            ("512x512 Euler with source field", [SourceProblem(steps=10).case])]
    out = {}
    for name, cs in work:
        row = {}
        for threads in (allc, 1):
            oracle.set_threads(threads)
            # size the sample on one step of the first grid
            o = oracle.Oracle(cs[0])
            U = cs[0].U0.copy()
            t0 = time.perf_counter()
            o.run(U, 0, 1)
            t1 = time.perf_counter() - t0
            o.close()
            per_case = t1 * sum(c.points for c in cs) / cs[0].points
            n = max(1, min(50, int(seconds / max(per_case, 1e-4))))
            pts = 0
            t0 = time.perf_counter()
            for c in cs:
                o = oracle.Oracle(c)
                U = c.U0.copy()
                o.run(U, 0, n)
                o.close()
                pts += c.points * n
            dt = time.perf_counter() - t0
            row[f"{threads}_cores" if threads > 1 else "1_core"] = {
                "value": pts / dt / 1e6, "steps_sampled": n}
        out[name] = row
    oracle.set_threads(allc)
    return {"unit": UNIT, "cores": allc, "kind": "port",
            "sample": "C oracle (-O3, OpenMP over lines), a few steps of each workload",
            "workloads": out}


def run_ours(args, world, rank, local, pg):
    import torch
    from navierstokes_gb300 import Solver
    from navierstokes_gb300 import _lib as L

    torch.cuda.set_device(local)
    case = build_case(args)
    solver = Solver(case, device=local)
    # a stream of our own: the legacy default stream (handle 0) is not one the
    # library can be handed, and events must sit on the launching stream
    stream = torch.cuda.Stream()
    solver.set_stream(stream.cuda_stream)
    solver.set_state(case.U0)
    launches = solver.launches_per_step()

    def barrier():
        if pg is not None:
            pg.barrier()

    for it in range(args.warmup):
        solver.step(it, 1)
    torch.cuda.synchronize()

    # ---- device-resident throughput -------------------------------------
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(args.steps):
        solver.step(args.warmup + k, 1)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = max_over_ranks(pg, ev0.elapsed_time(ev1), f"cuda:{local}")
    ms_step = ms / args.steps
    value = whole_job_rate(world, case.points, args.steps, ms * 1e-3)

    # ---- per-kernel device times (events around each launch) ---------------
    import ctypes as C
    kms = (C.c_double * L.NS_KC_COUNT)()
    kn = (C.c_int * L.NS_KC_COUNT)()
    L.check(solver.lib.ns_time_kernels(solver._ctx, 10_000, 2, kms, kn), solver._ctx)
    kernels = {}
    for k in range(L.NS_KC_COUNT):
        if kn[k]:
            name = solver.lib.ns_kernel_name(k).decode()
            kernels[name] = {"ms_per_launch": kms[k], "launches_per_step": kn[k],
                             "share": 0.0}
    tot = sum(v["ms_per_launch"] * v["launches_per_step"] for v in kernels.values())
    for v in kernels.values():
        v["share"] = v["ms_per_launch"] * v["launches_per_step"] / tot
    dom = max(kernels, key=lambda n: kernels[n]["share"])
    hbm_peak, peak_kind = load_peaks()
    dms = kernels[dom]["ms_per_launch"]
    bytes_launch = BYTES_PER_POINT.get(dom, 0) * case.points
    achieved = bytes_launch / (dms * 1e-3) / 1e9
    trafficpp = TRAFFIC_PER_POINT.get(dom)
    # The FP64 pipe binds every FP64 kernel (ncu: 83-89 % busy), so the
    # headline roofline is that pipe: FP64-pipe thread instructions per second
    # against the nominal 2 per clock per SM at the maximum SM clock.  The HBM
    # figures of the same kernel stand beside it.
    hbm = {"achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
           "bytes_per_launch": bytes_launch,
           "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"}
    traffic = trafficpp * case.points if trafficpp else None
    fp64_peak = C.c_double(0.0)
    if solver.lib.ns_fp64_peak(local, C.byref(fp64_peak)) != 0 or fp64_peak.value <= 0:
        fp64_peak.value = FP64_PEAK_FALLBACK_TFLOPS
    for name, v in kernels.items():
        fl = FP64_FLOP_PER_POINT.get(name)
        if fl:
            v["fp64_tflops"] = fl * case.points / (v["ms_per_launch"] * 1e-3) / 1e12
            v["fp64_frac"] = v["fp64_tflops"] / fp64_peak.value
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    sm_max_mhz = clocks.get("sm_max_mhz") or 2070.0
    nominal_ins = 2.0 * nsm * sm_max_mhz * 1e6
    ins = FP64_INST_PER_POINT[dom] * case.points / (dms * 1e-3)
    tf = FP64_FLOP_PER_POINT[dom] * case.points / (dms * 1e-3) / 1e12
    roof = {"bound": "fp64", "kernel": dom,
            "achieved": ins / 1e9, "peak": nominal_ins / 1e9, "unit": "FP64-pipe Ginst/s",
            "frac": ins / nominal_ins,
            "peak_source": f"nominal: 2 FP64 thread instructions per clock per SM, {nsm} SMs "
                           f"at {sm_max_mhz:.0f} MHz",
            "inst_per_point": FP64_INST_PER_POINT[dom],
            "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read+write per point of a 2048x2048 capture, "
                              "times the points of this launch",
            "hbm": hbm,
            "fp64_flops": {"achieved": tf, "unit": "TFLOP/s",
                           "flop_per_point": FP64_FLOP_PER_POINT[dom],
                           "dfma_loop_peak": fp64_peak.value,
                           "frac_of_dfma_loop": tf / fp64_peak.value,
                           "peak_source": "ns_fp64_peak(): DFMA loop measured live on this GPU"},
            "step": {"fp64_pipe_frac": FP64_INST_PER_POINT_STEP * case.points
                     / (ms_step * 1e-3) / nominal_ins,
                     "hbm_frac_fused_min": STEP_BYTES_FUSED_MIN * case.points
                     / (ms_step * 1e-3) / 1e9 / hbm_peak}}

    # ---- end to end through the C ABI with host buffers -----------------
    Uh = torch.empty(case.U0.shape, dtype=torch.float64, pin_memory=True).numpy()
    Uh[...] = case.U0
    solver.set_stream(0)
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        solver.rk_euler(Uh, (k + 1) * case.dt, k)
    t_e2e = max_over_ranks(pg, time.perf_counter() - t0, f"cuda:{local}")
    e2e_val = whole_job_rate(world, case.points, args.steps, t_e2e)
    nbytes = case.state_bytes()

    split = None
    if rank == 0 and world == 1 and not args.no_split:
        try:
            split = split_study(args, local, hbm_peak)
        except Exception as e:
            split = {"failed": str(e)}

    split_ns = None
    if rank == 0 and world == 1 and not args.no_split:
        try:
            split_ns = split_ns_study(args, local, hbm_peak)
        except Exception as e:
            split_ns = {"failed": str(e)}

    small = None
    if rank == 0 and world == 1 and not args.no_small_grid:
        try:
            small = small_grid_study(local)
        except Exception as e:
            small = {"failed": str(e)}

    batched = None
    if rank == 0 and world == 1 and not args.no_batch:
        try:
            batched = batch_study(args, local)
        except Exception as e:
            batched = {"failed": str(e)}

    adjoint = None
    if rank == 0 and world == 1 and not args.no_adjoint:
        try:
            adjoint = adjoint_study(args, local)
        except Exception as e:
            adjoint = {"failed": str(e)}

    cpu_workloads = None
    if rank == 0 and world == 1 and args.cpu_workloads:
        try:
            cpu_workloads = cpu_workloads_study()
        except Exception as e:
            cpu_workloads = {"failed": str(e)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline_sample(case)
        except Exception as e:  # the baseline must not kill the line
            cpu = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}
    solver.close()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64",
                "data": "synthetic: analytic pulse + isentropic vortex on the stretched grid",
                "config": workload_config(case),
                "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": nbytes,
                        "d2h_bytes_per_step": nbytes,
                        "call": "ns_rk_euler (host U(nk,imax,jmax) in/out, one step per call)"},
                "gpu_launches": launches * args.steps,
                "roofline": roof, "kernels": kernels, "clocks": clocks}
        if cpu is not None:
            line["cpu_baseline"] = cpu
        if split is not None:
            line["split_precision"] = split
        if split_ns is not None:
            line["split_precision_ns"] = split_ns
        if small is not None:
            line["small_grid"] = small
        if batched is not None:
            line["batched"] = batched
        if adjoint is not None:
            line["adjoint"] = adjoint
        if cpu_workloads is not None:
            line["cpu_workloads"] = cpu_workloads
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--imax", type=int, default=4096)
    ap.add_argument("--jmax", type=int, default=2048)
    ap.add_argument("--nk", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-split", action="store_true",
                    help="skip the split-precision study (Euler 4096^2)")
    ap.add_argument("--split-n", type=int, default=4096)
    ap.add_argument("--split-ns-steps", type=int, default=200,
                    help="steps of the Navier-Stokes split-precision comparison")
    ap.add_argument("--no-small-grid", action="store_true",
                    help="skip the 201x201 Euler pulse timing")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the batched-sweep study (64 instances)")
    ap.add_argument("--batch-n", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=300)
    ap.add_argument("--no-adjoint", action="store_true",
                    help="skip the discrete-adjoint study (512^2, 2000 steps)")
    ap.add_argument("--cpu-workloads", action="store_true",
                    help="also time the C oracle on every workload (all cores, 1 core)")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--adjoint-k", type=int, default=100,
                    help="adjoint checkpoint interval (the workload's 100); 0 keeps every stage "
                         "input if it fits")
    ap.add_argument("--split-error-steps", type=lambda t: [int(x) for x in t.split(",")],
                    default=[100, 500, 1000])
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        from navierstokes_gb300 import _build
        _build.build()
        run_ours(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
