#!/usr/bin/env python
"""Bench: time steps/s of the Bio-CFD hot path on one GB300.

Workload (one "step" = one time step of app/main.F90:129-265 over all blocks):
the two-block refinement case -- coarse 96x64x64 over 3x2x2 plus a nested
fine 64^3 block at ratio 2 around a stationary sphere D = 0.5, Re = 300,
uniform inflow, seeded N(0, 1e-3) noise, dt from CFL 0.3, SOR to 1e-6.

Three GPU paths run on the same GPU, each from the same initial state:
  * "fp64_dropin": FP64 red-black SOR with the reference's stop test
    (max |pc - pco| < 1e-6 every 5th iteration), bit-identical to the
    reference arithmetic;
  * "fp64": plain FP64 red-black SOR (FP64 momentum) run until the FP64
    Poisson residual in divergence units, dt * max|b/dt - A pc|, is <= 1e-6;
  * "mixed" (the flagship, reported as `value`): FP32 momentum stencil and
    FP32 red-black SOR inside an FP64 defect-correction loop, stopped at the
    same FP64 residual 1e-6 (so both end at equal divergence residual).
`e2e` repeats the flagship through the C ABI with host buffers: every step
uploads u,v,w,p of both blocks from pinned host memory and downloads them.
The CPU baseline is the serial FP64 oracle (the reference itself is Fortran
and no Fortran compiler exists on either machine).
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

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "bio-cfd_gb300"))
sys.path.insert(0, str(ROOT))

DIV_TOL = 1e-6
METRIC = "time steps/s at 1e-6 div residual: FP32+FP64-refine vs plain FP64, same GPU"
WORKLOAD = "two-block sphere: coarse 96x64x64 over 3x2x2 + fine 64^3 at ratio 2, D=0.5, Re=300"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def traffic_from_profiles():
    """dram read+write bytes per launch of the dominant kernel, from the committed ncu summary."""
    f = ROOT / "profiles" / "k_sor_dc_two_block.md"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for q, n in enumerate(names):
                if len(r) > 5 + q and r[5 + q].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), \
        int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(values):
    """Each value's maximum over the ranks of the process group (the values of
    this process when no group is initialised).  Replicas only: this all-reduce
    of a few timings is the sole collective."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def rank_barrier(torch):
    """Barrier over the replicas (when a group exists) and a device synchronize."""
    import torch.distributed as dist
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
    if torch.cuda.is_available():
        torch.cuda.synchronize()


def oracle_steps(case, n_steps: int):
    """Serial FP64 oracle (CPU): steps/s over n_steps steps after set-up."""
    from oracle.bridge import Oracle
    o = Oracle(checked=False)
    o.setup(case)
    t0 = time.perf_counter()
    for _ in range(n_steps):
        o.step()
    dt = time.perf_counter() - t0
    return n_steps / dt, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from biocfd import synth
    case = synth.sphere_two_block(n_steps=args.steps)
    # bounded sample: warm-up and timed steps of the serial oracle, capped so
    # the whole run stays within a few minutes
    k = max(1, min(args.steps, 6))
    sps, secs = oracle_steps(case, k)
    line = {"metric": METRIC, "value": sps, "unit": "steps/s", "n_gpus": 0, "steps": k,
            "warmup": 0, "ms_per_step": 1000.0 / sps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, numpy default_rng 20261203)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "precision": "fp64 serial oracle"},
            "cpu_baseline": {"value": sps, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": f"{k} time steps of the workload on the serial FP64 oracle "
                                       f"(the Fortran reference is unbuildable: no Fortran compiler), {secs:.1f} s"},
            "e2e": {"value": sps, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_path(solver, torch, flush, stream, steps: int, warmup: int, precision: int, div_tol: float,
              clocks: "Clocks | None" = None):
    """Per-step CUDA-event timing on the library stream, L2 flushed between
    steps; each step is a replay of the captured step graph.  One more step
    afterwards runs inside the profiling window (kernel by kernel) for the
    solve's device time and algorithmic bytes."""
    for _ in range(warmup):
        solver.run(1, precision=precision, div_tol=div_tol, use_graph=1)
    times, divs, res, iters = [], [], [], []
    ctx = clocks if clocks is not None else _Null()
    k0 = solver.kernel_launches()
    rank_barrier(torch)
    with ctx:
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            solver.run(1, precision=precision, div_tol=div_tol, use_graph=1)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            d = [solver.divergence(g) for g in solver.handles]
            divs.append(max(x[0] for x in d))
            res.append(max(x[1] for x in d))
            iters.append([solver.sor_stats(g)[0] for g in solver.handles])
    rank_barrier(torch)
    launches = solver.kernel_launches() - k0
    solver.profile_begin()
    solver.run(1, precision=precision, div_tol=div_tol)
    prof = solver.profile_end()
    prof["timed_launches"] = launches
    return times, divs, res, iters, prof


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def sweep_roofline(torch, local, hbm, block=(384, 256, 256), fp32_pairs=40, fp64_pairs=4):
    """Poisson sweeps on one body-free 384x256x256 block (the coarse block of
    the tandem-plate workload, ~25M cells, far above the 129 MB L2): achieved
    GB/s of the FP32 and FP64 red-black sweep kernels, algorithmic bytes from
    the solve log (17 B / 33 B per cell per sweep pair plus the FP64 residual
    and update passes of the FP32 correction)."""
    from biocfd import synth
    from biocfd.solver import Solver
    from biocfd._lib import check
    case = synth.uniform_block(tuple(block), noise=True)
    s = Solver(case, device=local)
    s.setup()
    g = s.handles[0]
    check(s.L.bcfd_cellcount_solid(g), "cellcount_solid")
    check(s.L.bcfd_compute_div(g), "compute_div")
    check(s.L.bcfd_block_sor_sweeps(g, 2, 1), "sor_sweeps")
    s.autotune()  # the launch shapes a user gets after bcfd_autotune
    cells = block[0] * block[1] * block[2]
    out = {"block": "x".join(map(str, block)) + f" ({cells / 1e6:.1f}M cells), no body",
           "l2": f"FP32 working set {17 * cells / 1e6:.0f} MB vs 129 MB L2",
           "solve_launch": s.solve_launch(g)}
    for prec, pairs, key in ((1, fp32_pairs, "fp32"), (0, fp64_pairs, "fp64")):
        if pairs <= 0:
            continue
        runs = {}
        for n in (pairs, 2 * pairs):
            s.profile_begin()
            check(s.L.bcfd_block_sor_sweeps(g, n, prec), "sor_sweeps")
            runs[n] = s.profile_end()
        p = runs[pairs]
        gbs = p["sor_bytes"] / (p["sor_ms"] * 1e-3) / 1e9
        # the sweep pairs alone: the difference between the 2P and P launches
        # (the residual, update and launch costs cancel)
        q = runs[2 * pairs]
        mgbs = (q["sor_bytes"] - p["sor_bytes"]) / ((q["sor_ms"] - p["sor_ms"]) * 1e-3) / 1e9
        out[key] = {"sweep_pairs": pairs, "ms": p["sor_ms"], "gbs": gbs, "frac_of_measured_hbm": gbs / hbm,
                    "bytes": p["sor_bytes"], "sweep_pair_gbs_marginal": mgbs,
                    "sweep_pair_frac_of_measured_hbm": mgbs / hbm,
                    "half_sweep_us": (q["sor_ms"] - p["sor_ms"]) * 1e3 / (2 * pairs)}
    s.close()
    return out


def twelve_block(torch, local, steps=10, warmup=3, fp64_steps=2, moving=False):
    """Twelve uneven blocks (coarse 256x192x192 + 11 fine blocks, 13.3M cells,
    stationary thin plate): mixed-path time per step with the batched launches
    and with one launch per block, and the plain FP64 path to the same residual.
    The working set (> 2 GB) is far above L2, so no flush is needed."""
    from biocfd import synth
    from biocfd.solver import Solver
    case = synth.twelve_block(n_steps=steps + warmup + 2, moving=moving)
    ncells = sum(b.nx * b.ny * b.nz for b in case.blocks)
    body = case.blocks[1]
    out = {"workload": "12 blocks: coarse 256x192x192 over 8x6x6 + 11 fine blocks at ratio 2 "
                       f"({body.nx}x{body.ny}x{body.nz} with a plate 0.5x0.125x0.0125, 2x128x64x64, 2x96x64x64, "
                       f"2x64x48x48, 2x48^3, 2x32^3), {ncells / 1e6:.1f}M cells, Re 500" +
                       (", plate heaving 0.5 sin(2 pi 0.25 t) and pitching 30 deg sin(2 pi 0.25 t + 90 deg), "
                        "Search every step, graph replay (each step's kinematics staged before its launch)" if moving else
                        ", stationary plate, graph replay"),
           "div_tol": DIV_TOL}
    arms = (("mixed_batched", 1, True, steps), ("mixed_per_block", 1, False, steps),
            ("fp64_batched", 2, True, fp64_steps))
    for key, prec, batching, n in arms:
        if n <= 0:
            continue
        s = Solver(case, device=local)
        s.set_batching(batching)
        s.setup()
        s.autotune()
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        for _ in range(warmup if prec == 1 else 1):
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
        ts = []
        k0 = s.kernel_launches()
        for _ in range(n):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        res = max(s.divergence(g)[1] for g in s.handles)
        ms = statistics.mean(ts)
        out[key] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "steps": n, "div_residual": res,
                    "launches_per_step": (s.kernel_launches() - k0) / n,
                    "cell_updates_per_s": ncells * 1000.0 / ms}
        s.close()
    if "fp64_batched" in out:
        out["speedup_mixed_vs_fp64"] = out["fp64_batched"]["ms_per_step"] / out["mixed_batched"]["ms_per_step"]
    out["speedup_batched_vs_per_block"] = (out["mixed_per_block"]["ms_per_step"] /
                                           out["mixed_batched"]["ms_per_step"])
    return out


def tandem(torch, local, steps=5, warmup=2, cmp_steps=2, moving=False):
    """Two stationary plates in tandem on the 45M-cell layout (coarse 384x256x256
    + two fine 256x192x192 blocks): time per step of the mixed path to the
    divergence residual 1e-6, of the plain FP64 path with the input's omega 1.7
    (which stops at pcItaMax = 5000 iterations per solve on the 384-cell block,
    short of 1e-6) and of the plain FP64 path relaxing with the mixed path's
    factor (which reaches 1e-6); and the mixed path's error against both FP64
    runs after `cmp_steps` steps from the same initial state (relative L2 of
    u, v, w, p per block; the drag and lift coefficients of each plate).
    With `moving` (both plates heaving and pitching, Search every step) only
    the mixed path and the FP64 path at the mixed path's factor run."""
    import numpy as np
    from biocfd import synth
    from biocfd.solver import Solver
    assert cmp_steps >= 2
    case = synth.tandem_plates(n_steps=steps + warmup + cmp_steps + 2, moving=moving)
    ncells = sum(b.nx * b.ny * b.nz for b in case.blocks)
    out = {"workload": "tandem plates: coarse 384x256x256 over 6x4x4 + two fine 256x192x192 at ratio 2, "
                       f"{ncells / 1e6:.1f}M cells, " +
                       ("plates heaving 0.125 sin(2 pi 0.25 t) and pitching 15 deg sin(2 pi 0.25 t + 90 deg), "
                        "Search every step, " if moving else "stationary ") +
                       "plates 0.5x0.125x0.0125 with centres 2.5 apart (1.5 chords), Re 1000, graph replay",
           "div_tol": DIV_TOL}
    mu_f = 1.0 / case.re
    snaps = {}
    case_om = synth.with_mixed_omega(case)
    arms = [("mixed", 1, steps, case), ("fp64", 2, 1, case), ("fp64_mixed_omega", 2, 1, case_om)]
    if moving:
        del arms[1]
    for key, prec, n_timed, arm_case in arms:
        s = Solver(arm_case, device=local)
        s.setup()
        s.autotune()
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        # mixed: cmp_steps, warm-up, then the timed steps; FP64: cmp_steps, the
        # last of them (a graph replay) timed
        n_pre = cmp_steps + warmup if prec == 1 else cmp_steps - 1
        ts = []
        k0 = 0
        for it in range(n_pre + n_timed):
            timed = it >= n_pre
            if it == n_pre:
                k0 = s.kernel_launches()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
            e1.record(stream)
            e1.synchronize()
            if timed:
                ts.append(e0.elapsed_time(e1))
            if it == cmp_steps - 1:
                snaps[key] = ([s.fields(g) for g in s.handles],
                              [s.stress(g, mu_f).tolist() for g in s.handles[1:]])
        res = max(s.divergence(g)[1] for g in s.handles)
        ms = statistics.mean(ts)
        out[key] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "steps": len(ts), "div_residual": res,
                    "launches_per_step": (s.kernel_launches() - k0) / len(ts),
                    "cell_updates_per_s": ncells * 1000.0 / ms}
        s.close()
    out["fp64_mixed_omega"]["omega"] = [b.omega for b in case_om.blocks]
    if "fp64" in out:
        out["fp64"]["omega"] = [b.omega for b in case.blocks]
        out["speedup_mixed_vs_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    out["speedup_mixed_vs_fp64_mixed_omega"] = (out["fp64_mixed_omega"]["ms_per_step"] /
                                                out["mixed"]["ms_per_step"])
    fm, sm = snaps["mixed"]
    for ref in ("fp64_mixed_omega", "fp64"):
        if ref not in snaps:
            continue
        fd, sd = snaps[ref]
        err = {}
        for q in range(len(fm)):
            for k in ("u", "v", "w", "p"):
                a, b = fm[q][k], fd[q][k]
                if k == "p":  # pressure is defined up to a constant per solve: compare about the mean
                    a, b = a - a.mean(), b - b.mean()
                err[f"block{q + 1}_{k}"] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
        out[f"error_vs_{ref}"] = {"after_steps": cmp_steps, "field_rel_l2": err,
                                  "coefficients": "viscous drag, pressure drag, viscous lift, pressure lift",
                                  "plates_mixed": sm, f"plates_{ref}": sd,
                                  "coef_rel": [[abs(x - y) / max(abs(y), 1e-300) for x, y in zip(a, b)]
                                               for a, b in zip(sm, sd)]}
    return out


def adjoint_bench(torch, local, steps=4, every=2):
    """Discrete adjoint of whole FP64 steps on the 64^3 sphere block (D = 0.25,
    Re 100): time per step of forward + checkpointed reverse pass for the
    objective "time-averaged drag + lift coefficients", with the adjoint
    Poisson solves in FP64 SOR and in FP32 sweeps + FP64 defect correction
    (both to the same FP64 residual)."""
    import time
    from biocfd import synth
    from biocfd.adjoint import adjoint_run
    from biocfd.solver import Solver
    case = synth.sphere_single_block(n=64, n_steps=steps + 2)
    out = {"workload": f"64^3 sphere block (D=0.25, Re 100), {steps} FP64 steps, checkpoint every {every}, "
                       "objective mean of drag + lift coefficients, gradients in uc, u,v,w,p^0 and the "
                       "body's kinematic scalars", "adj_tol": 1e-13}
    for key, prec in (("adjoint_fp64_solves", 0), ("adjoint_mixed_solves", 1)):
        s = Solver(case, device=local)
        s.setup()
        s.run(1)  # the per-step re-Search settles the tags of the set-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        J, duc, g = adjoint_run(s, {}, steps, every=every, stress_seed=(1.0, 1.0, 0.0, 0.0),
                                mu_f=1.0 / case.re, rho_f=1.0, adj_tol=1e-13, solve_precision=prec)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        out[key] = {"ms_per_step": 1000.0 * secs / steps, "J": J, "dJ_duc": duc}
        s.close()
    out["speedup_mixed_solves"] = (out["adjoint_fp64_solves"]["ms_per_step"] /
                                   out["adjoint_mixed_solves"]["ms_per_step"])
    out["dJ_duc_rel_diff"] = abs(out["adjoint_fp64_solves"]["dJ_duc"] - out["adjoint_mixed_solves"]["dJ_duc"]) / \
        abs(out["adjoint_fp64_solves"]["dJ_duc"])
    return out


def run_gpu(args):
    import numpy as np
    import torch
    from biocfd import synth
    from biocfd.solver import Solver

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    case = synth.sphere_two_block(n_steps=args.steps + args.warmup)
    s = Solver(case, device=local)
    s.setup()
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    tol = DIV_TOL

    if args.mixed_only:
        # the flagship arm alone (for profiler captures of its kernels)
        s.autotune()
        t, _, res, it, _ = time_path(s, torch, flush, stream, args.steps, args.warmup, 1, tol)
        print(json.dumps({"run": "mixed arm only", "ms_per_step": statistics.mean(t), "div_residual": max(res),
                          "fp32_sweeps_last_step": it[-1]}), flush=True)
        s.close()
        return

    def arm(precision, clocks=None, arm_case=None):
        nonlocal s, stream
        s.close()
        s = Solver(case if arm_case is None else arm_case, device=local)
        s.setup()
        s.autotune()  # launch shapes of the solves; results do not depend on them
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        return time_path(s, torch, flush, stream, args.steps, args.warmup, precision, tol, clocks)

    # drop-in FP64 path: the reference's stop test (max|pc - pco| < 1e-6)
    t0_, div0, res0, it0, prof0 = arm(0)
    # plain FP64 SOR run to the same FP64 residual target as the mixed path
    t64, div64, res64, it64, prof64 = arm(2)
    # the same, relaxing with the mixed path's factor instead of the input's 1.7
    case_om = synth.with_mixed_omega(case)
    t64o, _, res64o, it64o, _ = arm(2, arm_case=case_om)
    # flagship: FP32 momentum + FP32 SOR with FP64 defect correction
    clocks = Clocks(local)
    tmx, divmx, resmx, itmx, profmx = arm(1, clocks)
    # e2e through the C ABI with host buffers (pinned), flagship precision
    host = []
    for spec, g in zip(case.blocks, s.handles):
        f = s.fields(g)
        host.append({k: torch.from_numpy(np.ascontiguousarray(f[k].ravel(order="F"))).pin_memory()
                     for k in ("u", "v", "w", "p")})
    import ctypes as C
    from biocfd._lib import P_d, check
    nbytes = sum(h[k].numel() * 8 for h in host for k in ("u", "v", "w", "p"))
    e2e_times = []
    for step in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for h, g in zip(host, s.handles):
            ptr = [C.cast(h[k].data_ptr(), P_d) for k in ("u", "v", "w", "p")]
            check(s.L.bcfd_block_upload_fields(g, *ptr, None, None, None), "upload")
        s.run(1, precision=1, div_tol=tol, use_graph=1)
        for h, g in zip(host, s.handles):
            ptr = [C.cast(h[k].data_ptr(), P_d) for k in ("u", "v", "w", "p")]
            check(s.L.bcfd_block_download_fields(g, *ptr, None, None, None), "download")
        e2e_times.append(time.perf_counter() - t0)

    ms64 = statistics.mean(t64)
    ms64o = statistics.mean(t64o)
    ms0 = statistics.mean(t0_)
    msmx = statistics.mean(tmx)
    e2e_s = statistics.mean(e2e_times)
    msmx, ms64, ms0, e2e_s, ms64o = max_over_ranks([msmx, ms64, ms0, e2e_s, ms64o])
    nfluid = sum(s.counts(g)["fluidCellCount"] for g in s.handles)
    hbm, peak_kind = peaks()
    achieved = profmx["sor_bytes"] / (profmx["sor_ms"] * 1e-3) / 1e9 if profmx["sor_ms"] > 0 else 0.0
    ach64 = prof64["sor_bytes"] / (prof64["sor_ms"] * 1e-3) / 1e9 if prof64["sor_ms"] > 0 else 0.0
    traffic = traffic_from_profiles()
    line = {
        "metric": METRIC,
        "value": world * 1000.0 / msmx,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": msmx,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 sweeps + f64 defect correction",
        "data": "synthetic (seeded, numpy default_rng 20261203)",
        "config": {"workload": WORKLOAD, "blocks": "96x64x64 + 64^3", "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed steps (256 MB write)", "timed": "per-step CUDA events",
                   "launch": "each step one replay of the captured step CUDA graph"},
        "fp64": {"steps_per_s": 1000.0 / ms64, "ms_per_step": ms64, "div_residual": max(res64),
                 "div_tol": tol, "max_div_after_correction": max(div64), "sor_iters_last_step": it64[-1],
                 "solve_gbs": ach64},
        "fp64_dropin": {"steps_per_s": 1000.0 / ms0, "ms_per_step": ms0, "div_residual": max(res0),
                        "stop": "max|pc - pco| < epsi every 5th iteration (reference stop test)",
                        "sor_iters_last_step": it0[-1]},
        "mixed": {"steps_per_s": 1000.0 / msmx, "ms_per_step": msmx, "div_residual": max(resmx),
                  "div_tol": tol, "max_div_after_correction": max(divmx), "fp32_sweeps_last_step": itmx[-1]},
        "fp64_mixed_omega": {"steps_per_s": 1000.0 / ms64o, "ms_per_step": ms64o, "div_residual": max(res64o),
                             "omega": [b.omega for b in case_om.blocks], "sor_iters_last_step": it64o[-1],
                             "speedup_mixed_vs_this": ms64o / msmx,
                             "note": "plain FP64 SOR relaxing with the mixed path's default factor "
                                     "2/(1+sin(pi/n_max)) instead of the input's 1.7"},
        "speedup_vs_fp64": ms64 / msmx,
        "cell_updates_per_s": world * nfluid * 1000.0 / msmx,
        "e2e": {"value": world / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "gpu_launches": profmx["timed_launches"],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "kernel": "mixed Poisson solve (k_sor_dc or k_sor_tb, as autotuned)",
                     "peak_source": peak_kind,
                     "note": "algorithmic bytes: 17 B per cell per FP32 sweep pair + FP64 residual/update passes; "
                             "the 64^3 and 96x64x64 blocks are L2-resident during a solve"},
        "clocks": clocks.summary(),
        "solve_launch": {f"block{q + 1}": s.solve_launch(g) for q, g in enumerate(s.handles)},
    }
    if not args.no_sweep_roofline:
        line["sweep_roofline"] = sweep_roofline(torch, local, hbm)
    if not args.no_twelve_block:
        line["twelve_block"] = twelve_block(torch, local)
        line["twelve_block_moving"] = twelve_block(torch, local, steps=5, fp64_steps=1, moving=True)
    if not args.no_adjoint:
        line["adjoint"] = adjoint_bench(torch, local)
    if not args.no_tandem:
        line["tandem"] = tandem(torch, local)
        line["tandem_moving"] = tandem(torch, local, moving=True)
    if rank == 0 and not args.no_cpu_baseline:
        sps, secs = oracle_steps(case, 1)
        line["cpu_baseline"] = {"value": sps, "unit": "steps/s", "cores": 1, "kind": "port",
                                "sample": f"1 time step of the same workload on the serial FP64 oracle, {secs:.1f} s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    s.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sweep-roofline", action="store_true")
    ap.add_argument("--no-twelve-block", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-tandem", action="store_true")
    ap.add_argument("--tandem-only", action="store_true",
                    help="only the 45M-cell tandem-plate measurement (mixed vs FP64, error vs FP64)")
    ap.add_argument("--adjoint-only", action="store_true", help="only the adjoint timing")
    ap.add_argument("--twelve-only", action="store_true",
                    help="only the twelve-block measurement (batched vs per-block launches)")
    ap.add_argument("--mixed-only", action="store_true",
                    help="time only the flagship arm and print a short line (profiler captures)")
    ap.add_argument("--sweep-only", default="",
                    help="nx,ny,nz[,fp32_pairs[,fp64_pairs]]: only the Poisson sweep measurement on that block")
    args = ap.parse_args()
    if args.adjoint_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(adjoint_bench(torch, 0)), flush=True)
        return
    if args.tandem_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(tandem(torch, 0)), flush=True)
        print(json.dumps(tandem(torch, 0, moving=True)), flush=True)
        return
    if args.twelve_only:
        import torch
        print(json.dumps(twelve_block(torch, 0, args.steps, args.warmup)), flush=True)
        print(json.dumps(twelve_block(torch, 0, args.steps, args.warmup, fp64_steps=1, moving=True)), flush=True)
        return
    if args.sweep_only:
        import torch
        v = [int(x) for x in args.sweep_only.split(",")]
        hbm, _ = peaks()
        r = sweep_roofline(torch, 0, hbm, v[:3], v[3] if len(v) > 3 else 40, v[4] if len(v) > 4 else 4)
        print(json.dumps(r), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
