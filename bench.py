#!/usr/bin/env python
"""Bench: time steps/s of the Bio-CFD hot path on one GB300.

Headline workload (one "step" = one time step of app/main.F90:129-265 over
all blocks): the largest single-GPU configuration, tandem flapping plates on
44.0M cells -- a coarse 384x256x256 block over 6x4x4 plus two fine
256x192x192 blocks at ratio 2, each holding a rigid ellipsoidal plate
(0.5 x 0.125 x 0.0125) 1.5 chords apart, Re = 1000; the leading plate heaves
0.125 sin(2 pi 0.25 t) and pitches 15 deg sin(2 pi 0.25 t + 90 deg), the
trailing plate does the same 90 deg behind; Search every step; seeded
N(0, 1e-3) noise on u = 1.

`value` is the flagship path: FP32 momentum stencil and FP32 red-black SOR
inside an FP64 defect-correction loop, every solve stopped at the FP64
Poisson residual dt * max|b/dt - A pc| <= 1e-6, each step one replay of the
captured step CUDA graph.  Beside it, on the same GPU and workload:
  * "fp64_fast": plain FP64 (FP64 momentum, FP64 SOR without divisions) to the
    same residual -- the metric's FP64 denominator;
  * "fp64": plain FP64 with the reference's sweep arithmetic to the same
    residual; "fp64_input_omega": the same with the input omega 1.7;
  * the per-phase split of one step, the roofline of the dominant kernel (the
    mixed Poisson solve), and the mixed path's error against the FP64 run.
`e2e` repeats the flagship through the C ABI with host buffers: every step
uploads u,v,w,p of all blocks from pinned host memory and downloads them.
The CPU baseline / reference arm is the FP64 oracle on the host cores (the
reference itself is Fortran and no Fortran compiler exists on either
machine), timed on a bounded sample of the same workload (see
`cpu_reference_sample`).
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
WORKLOAD = ("tandem flapping plates, 44.0M cells: coarse 384x256x256 over 6x4x4 + two fine 256x192x192 at "
            "ratio 2, plates 0.5x0.125x0.0125 1.5 chords apart heaving 0.125 sin(2 pi 0.25 t) and pitching "
            "15 deg sin(2 pi 0.25 t + 90 deg), trailing plate 90 deg behind, Re 1000, Search every step")

# Sweep pairs the reference algorithm (FP64 SOR, omega 1.7, stop when
# max|pc - pco| < 1e-6 every 5th iteration, at most pcItaMax = 5000 per solve)
# spends per block in the first step of the headline workload, summed over the
# block's solve calls in the step (the coarse block is solved once, each fine
# block twice).  Measured with the GPU drop-in path, whose iteration counts
# equal the oracle's bit for bit; the CPU reference arm multiplies its
# measured cost per sweep pair by these counts.
REFERENCE_SWEEP_PAIRS = (1400, 2645, 2560)  # coarse, fine 1, fine 2 (bench.py --dropin-steps 1)


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profile_value(name: str, key: str):
    """A `key: value` line of a committed ncu summary under profiles/."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except (ValueError, IndexError):
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
                                          "--format=csv,noheader,nounits", "-lms", "100"],
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


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False

    def summary(self):
        return None


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


# ---------------------------------------------------------------------------
# CPU reference: the FP64 oracle (all host threads) on a bounded sample
# ---------------------------------------------------------------------------

def cpu_reference_sample(case, sweep_pairs=None, cap_pairs: int = 4):
    """Time the oracle (the FP64 restatement of the reference; its OpenMP loops
    use every host core) on a bounded sample of one time step of `case` and
    return the estimated time of a whole reference step.

    The sample is one full time step with every Poisson solve capped at
    `cap_pairs` sweep pairs (pcItaMax), plus `cap_pairs` more sweep pairs of
    each block timed alone; a whole step then costs the capped step plus, per
    block, (the reference's sweep pairs - the capped ones) times the measured
    cost of one pair.  `sweep_pairs` are the reference's sweep pairs per block
    in that step (REFERENCE_SWEEP_PAIRS); without them the capped step alone
    is reported (a lower bound)."""
    from biocfd import synth
    from oracle.bridge import Oracle
    o = Oracle(checked=False)
    t0 = time.perf_counter()
    o.setup(synth.replace(case, pc_ita_max=cap_pairs - 1))
    t_setup = time.perf_counter() - t0
    threads = int(o.L.orc_get_threads())
    t0 = time.perf_counter()
    o.step()
    t_capped = time.perf_counter() - t0
    nb = len(case.blocks)
    capped_pairs = [o.geti(g, "nIterPcor") for g in range(1, nb + 1)]
    # per-block cost of one sweep pair: the block's SOR alone for cap_pairs pairs
    pair_s = []
    for g in range(1, nb + 1):
        o.seti(g, "nIterPcor", 0)
        t0 = time.perf_counter()
        o.L.orc_redblack_sor(g, cap_pairs - 1, case.dt, -1.0)
        pair_s.append((time.perf_counter() - t0) / max(o.geti(g, "nIterPcor"), 1))
    if sweep_pairs:
        extra = sum(max(n - c, 0) * t for n, c, t in zip(sweep_pairs, capped_pairs, pair_s))
        est = t_capped + extra
        how = (f"one oracle step with every Poisson solve capped at {cap_pairs} sweep pairs ({t_capped:.1f} s) "
               f"+ per block (the reference's sweep pairs {list(sweep_pairs)} - the capped ones {capped_pairs}) x "
               f"the block's measured seconds per sweep pair {[round(x, 4) for x in pair_s]}")
    else:
        est = t_capped
        how = f"one oracle step with every Poisson solve capped at {cap_pairs} sweep pairs (lower bound)"
    return {"step_s": est, "steps_per_s": 1.0 / est, "threads": threads, "sample": how,
            "setup_s": t_setup, "capped_step_s": t_capped, "pair_s": pair_s}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from biocfd import synth
    case = synth.tandem_plates(n_steps=2, moving=True)
    r = cpu_reference_sample(case, REFERENCE_SWEEP_PAIRS)
    # each of the K requested steps is this bounded sample; one sample
    # stands for all of them (the oracle is deterministic)
    line = {"metric": METRIC, "value": r["steps_per_s"], "unit": "steps/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * r["step_s"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded, numpy default_rng 20261203)", "impl": "reference",
            "config": {"workload": WORKLOAD, "precision": "FP64, the reference's algorithm (omega 1.7, "
                                                          "max|pc - pco| < 1e-6, pcItaMax 5000)"},
            "cpu_baseline": {"value": r["steps_per_s"], "unit": "steps/s", "cores": r["threads"], "kind": "port",
                             "sample": r["sample"] + "; FP64 oracle port (the Fortran reference is unbuildable "
                                       "here: no Fortran compiler on either machine)"},
            "e2e": {"value": r["steps_per_s"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arms
# ---------------------------------------------------------------------------

WARM_START = True  # residual-target solves start from the last correction (--zero-start turns it off)


def new_solver(case, local, tune=True, warm=None):
    from biocfd.solver import Solver
    s = Solver(case, device=local)
    s.setup()
    s.set_warm_start(WARM_START if warm is None else warm)
    if tune:
        s.autotune()  # launch shapes of the solves; results do not depend on them
    return s


def timed_steps(s, torch, steps, precision, clocks=None, graph=1):
    """Per-step CUDA events on the library stream; returns (ms list, launches)."""
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    ts = []
    k0 = s.kernel_launches()
    with (clocks if clocks is not None else _Null()):
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(1, precision=precision, div_tol=DIV_TOL, use_graph=graph)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
    return ts, s.kernel_launches() - k0


def profiled_step(s, precision):
    """One eager step inside a measurement window: solve device time and
    algorithmic bytes, kernels launched, and the per-phase device times."""
    s.profile_begin()
    s.run(1, precision=precision, div_tol=DIV_TOL)
    prof = s.profile_end()
    prof["phases_ms"] = s.profile_phases()
    return prof


def residual_stats(s):
    """Largest FP64 Poisson residual (divergence units) left by the last
    solves, and each block's SOR sweep pairs in the last step."""
    res = max(s.divergence(g)[1] for g in s.handles)
    return res, [s.sor_stats(g)[0] for g in s.handles]


def field_errors(fa, fb, sa, sb):
    import numpy as np
    err = {}
    for q in range(len(fa)):
        for k in ("u", "v", "w", "p"):
            a, b = fa[q][k], fb[q][k]
            if k == "p":  # pressure is defined up to a constant per solve: compare about the mean
                a, b = a - a.mean(), b - b.mean()
            err[f"block{q + 1}_{k}"] = float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
    coef = [[abs(x - y) / max(abs(y), 1e-300) for x, y in zip(a, b)] for a, b in zip(sa, sb)]
    return err, coef


def headline(args, torch, local, world):
    """The flagship mixed path on the tandem-plate workload, its FP64 arms,
    phase split, roofline and e2e."""
    import ctypes as C
    import numpy as np
    from biocfd import synth
    from biocfd._lib import P_d, check
    hbm, peak_kind = peaks()
    n_pre = 2  # steps every arm runs from the initial state before the compared state
    case = synth.tandem_plates(n_steps=args.steps + args.warmup + 8, moving=True)
    ncells = sum(b.nx * b.ny * b.nz for b in case.blocks)
    mu_f = 1.0 / case.re
    out = {}
    # ---- flagship: mixed precision --------------------------------------------
    t0 = time.perf_counter()
    s = new_solver(case, local)
    setup_s = time.perf_counter() - t0
    for _ in range(n_pre):
        s.run(1, precision=1, div_tol=DIV_TOL, use_graph=1)
    snap_mixed = ([s.fields(g) for g in s.handles], [s.stress(g, mu_f).tolist() for g in s.handles[1:]])
    for _ in range(args.warmup):
        s.run(1, precision=1, div_tol=DIV_TOL, use_graph=1)
    clocks = Clocks(local)
    rank_barrier(torch)
    tmx, launches = timed_steps(s, torch, args.steps, 1, clocks)
    rank_barrier(torch)
    res_mx, pairs_mx = residual_stats(s)
    prof = profiled_step(s, 1)
    nfluid = sum(s.counts(g)["fluidCellCount"] for g in s.handles)
    # ---- e2e through the C ABI with host buffers ------------------------------
    host = []
    for g in s.handles:
        f = s.fields(g)
        host.append({k: torch.from_numpy(np.ascontiguousarray(f[k].ravel(order="F"))).pin_memory()
                     for k in ("u", "v", "w", "p")})
    nbytes = sum(h[k].numel() * 8 for h in host for k in ("u", "v", "w", "p"))
    e2e_times = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for h, g in zip(host, s.handles):
            ptr = [C.cast(h[k].data_ptr(), P_d) for k in ("u", "v", "w", "p")]
            check(s.L.bcfd_block_upload_fields(g, *ptr, None, None, None), "upload")
        s.run(1, precision=1, div_tol=DIV_TOL, use_graph=1)
        for h, g in zip(host, s.handles):
            ptr = [C.cast(h[k].data_ptr(), P_d) for k in ("u", "v", "w", "p")]
            check(s.L.bcfd_block_download_fields(g, *ptr, None, None, None), "download")
        e2e_times.append(time.perf_counter() - t0)
    solve_launch = {f"block{q + 1}": s.solve_launch(g) for q, g in enumerate(s.handles)}
    s.close()
    msmx = statistics.mean(tmx)
    e2e_s = statistics.mean(e2e_times)
    msmx, e2e_s = max_over_ranks([msmx, e2e_s])
    achieved = prof["sor_bytes"] / (prof["sor_ms"] * 1e-3) / 1e9 if prof["sor_ms"] > 0 else 0.0
    out["mixed"] = {"ms_per_step": msmx, "steps_per_s": 1000.0 / msmx, "steps": len(tmx),
                    "div_residual": res_mx, "sweep_pairs_last_step": pairs_mx,
                    "cell_updates_per_s": nfluid * 1000.0 / msmx, "launches_per_step": launches / len(tmx),
                    "setup_s": setup_s, "solve_launch": solve_launch}
    step_ms = sum(prof["phases_ms"].values())
    out["phases"] = {"ms": prof["phases_ms"],
                     "share": {k: v / step_ms for k, v in prof["phases_ms"].items()} if step_ms > 0 else {},
                     "note": "one eagerly issued step of the flagship path (CUDA events at phase boundaries on "
                             "the library stream); its total exceeds a graph replay by the launch gaps"}
    # DRAM bytes per launch: the ratio of DRAM traffic to algorithmic bytes of
    # the solve launches of one step of this workload (one ncu capture, the
    # committed summary) times this run's algorithmic bytes per launch
    ratio = profile_value("k_sor_dc_tandem_dram.md", "traffic_over_algorithmic")
    per_launch = prof["sor_bytes"] / prof["sor_launches"] if prof["sor_launches"] else 0.0
    traffic = ratio * per_launch if ratio is not None else None
    out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                       "frac": achieved / hbm, "traffic": traffic,
                       "traffic_over_algorithmic": ratio,
                       "kernel": "mixed Poisson solve launches (k_sor_dc / k_sor_dc_set, as autotuned)",
                       "peak_source": peak_kind,
                       "launches": prof["sor_launches"], "ms": prof["sor_ms"], "bytes": prof["sor_bytes"],
                       "note": "algorithmic bytes from the solve log: 17 B per cell per FP32 sweep pair, 29 B per "
                               "FP64 residual pass, 25 B per FP64 update pass; CUDA events around each solve "
                               "launch; the coarse block's FP32 working set (428 MB) streams from DRAM, the fine "
                               "blocks' (160 MB each, solved one at a time) mostly stays in the 129 MB L2, hence "
                               "traffic below the algorithmic bytes"}
    out["e2e"] = {"value": world / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": nbytes,
                  "d2h_bytes_per_step": nbytes}
    out["gpu_launches"] = launches
    out["clocks"] = clocks.summary()
    out["nfluid"] = nfluid
    out["ncells"] = ncells
    # ---- FP64 arms on the same workload ---------------------------------------
    case_om = synth.with_mixed_omega(case)
    arms = [("fp64_fast", 3, case_om, args.fp64_steps, "FP64 momentum + FP64 SOR without divisions (fused "
             "residual, Newton-Raphson inverse diagonal), relaxing with the mixed path's factor"),
            ("fp64", 2, case_om, args.fp64_steps, "FP64 momentum + FP64 SOR with the reference's sweep "
             "arithmetic (one IEEE division per update), relaxing with the mixed path's factor")]
    if args.fp64_input_omega:
        arms.append(("fp64_input_omega", 2, case, 1, "as fp64, relaxing with the input's omega 1.7"))
    for key, prec, arm_case, n_timed, what in arms:
        if n_timed <= 0:
            continue
        s = new_solver(arm_case, local)
        for _ in range(n_pre):
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
        snap = ([s.fields(g) for g in s.handles], [s.stress(g, mu_f).tolist() for g in s.handles[1:]])
        ts, nl = timed_steps(s, torch, n_timed, prec)
        res, pairs = residual_stats(s)
        s.close()
        ms = max_over_ranks([statistics.mean(ts)])[0]
        err, coef = field_errors(snap_mixed[0], snap[0], snap_mixed[1], snap[1])
        out[key] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "steps": len(ts), "div_residual": res,
                    "sweep_pairs_last_step": pairs, "omega": [b.omega for b in arm_case.blocks],
                    "what": what, "speedup_mixed_vs_this": ms / msmx,
                    "mixed_error_vs_this": {"after_steps": n_pre, "field_rel_l2": err,
                                            "coef_rel": coef,
                                            "coefficients": "per plate: viscous drag, pressure drag, viscous "
                                                            "lift, pressure lift"}}
    if WARM_START and args.zero_start_steps > 0:
        # the flagship with the reference's zero start of every solve
        s = new_solver(case, local, warm=False)
        for _ in range(n_pre + 1):
            s.run(1, precision=1, div_tol=DIV_TOL, use_graph=1)
        ts, _ = timed_steps(s, torch, args.zero_start_steps, 1)
        res, pairs = residual_stats(s)
        s.close()
        ms = statistics.mean(ts)
        out["mixed_zero_start"] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "steps": len(ts),
                                   "div_residual": res, "sweep_pairs_last_step": pairs,
                                   "note": "the flagship with every solve started from pc = 0, as the reference"}
    if args.dropin_steps > 0:
        # the drop-in path (reference arithmetic and stop test) on the same
        # workload: its sweep pairs are the reference's (REFERENCE_SWEEP_PAIRS)
        s = new_solver(case, local)
        ts, _ = timed_steps(s, torch, args.dropin_steps, 0, graph=0)
        out["fp64_dropin"] = {"ms_per_step": statistics.mean(ts), "steps": len(ts),
                              "sweep_pairs_per_step": [s.sor_stats(g)[0] for g in s.handles],
                              "stop": "max|pc - pco| < 1e-6 every 5th iteration, omega 1.7, pcItaMax 5000"}
        s.close()
    return out


def two_block(torch, local, steps, warmup):
    """The two-block sphere workload (coarse 96x64x64 over 3x2x2 + fine 64^3 at
    ratio 2, D = 0.5, Re 300): mixed path vs the FP64 arms, L2 flushed
    between steps (its working set fits in L2)."""
    from biocfd import synth
    case = synth.sphere_two_block(n_steps=steps + warmup + 4)
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2
    out = {"workload": "two-block sphere: coarse 96x64x64 over 3x2x2 + fine 64^3 at ratio 2, D=0.5, Re=300",
           "l2": "flushed between timed steps (256 MB write)"}
    for key, prec, c in (("mixed", 1, case), ("fp64_fast", 3, synth.with_mixed_omega(case)),
                         ("fp64", 2, synth.with_mixed_omega(case)), ("fp64_input_omega", 2, case),
                         ("fp64_dropin", 0, case)):
        s = new_solver(c, local)
        stream = torch.cuda.ExternalStream(s.stream_ptr())
        for _ in range(warmup):
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
        ts = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        res, pairs = residual_stats(s)
        s.close()
        ms = statistics.mean(ts)
        out[key] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "div_residual": res,
                    "sweep_pairs_last_step": pairs}
    for key in ("fp64_fast", "fp64", "fp64_input_omega"):
        out[f"speedup_mixed_vs_{key}"] = out[key]["ms_per_step"] / out["mixed"]["ms_per_step"]
    return out


def sweep_roofline(torch, local, hbm, block=(384, 256, 256), fp32_pairs=40, fp64_pairs=8):
    """Poisson sweeps on one body-free 384x256x256 block (the coarse block of
    the tandem-plate workload, ~25M cells, far above the 129 MB L2): achieved
    GB/s of the FP32 and FP64 red-black sweep kernels, algorithmic bytes from
    the solve log (17 B / 33 B per cell per sweep pair plus the FP64 residual
    and update passes of the FP32 correction)."""
    from biocfd import synth
    from biocfd._lib import check
    case = synth.uniform_block(tuple(block), noise=True)
    s = new_solver(case, local, tune=False)
    g = s.handles[0]
    check(s.L.bcfd_cellcount_solid(g), "cellcount_solid")
    check(s.L.bcfd_compute_div(g), "compute_div")
    check(s.L.bcfd_block_sor_sweeps(g, 2, 1), "sor_sweeps")
    s.autotune()
    cells = block[0] * block[1] * block[2]
    out = {"block": "x".join(map(str, block)) + f" ({cells / 1e6:.1f}M cells), no body",
           "l2": f"FP32 working set {17 * cells / 1e6:.0f} MB vs 129 MB L2", "solve_launch": s.solve_launch(g)}
    tuned = s.solve_launch(g)
    for prec, pairs, key in ((1, fp32_pairs, "fp32"), (1, fp32_pairs, "fp32_tiled_neighbour_sync"),
                             (1, fp32_pairs, "fp32_zmarch_tma"), (0, fp64_pairs, "fp64_reference_sweeps"),
                             (2, fp64_pairs, "fp64_division_free")):
        # fp32: the autotuned variant; then the tiled sweeps with neighbour
        # sync (variant 3) and the z-marching TMA sweeps (variant 5) alone
        variant = {"fp32": tuned["fp32_variant"], "fp32_tiled_neighbour_sync": 3, "fp32_zmarch_tma": 5}.get(key)
        if variant is not None:
            s.set_mixed_params(variant=variant, block=g)
        runs = {}
        for n in (pairs, 2 * pairs):
            s.profile_begin()
            check(s.L.bcfd_block_sor_sweeps(g, n, prec), "sor_sweeps")
            runs[n] = s.profile_end()
        p, q = runs[pairs], runs[2 * pairs]
        gbs = p["sor_bytes"] / (p["sor_ms"] * 1e-3) / 1e9
        # the sweep pairs alone: the difference between the 2P and P launches
        mgbs = (q["sor_bytes"] - p["sor_bytes"]) / ((q["sor_ms"] - p["sor_ms"]) * 1e-3) / 1e9
        pair_us = (q["sor_ms"] - p["sor_ms"]) * 1e3 / pairs
        out[key] = {"sweep_pairs": pairs, "ms": p["sor_ms"], "gbs": gbs, "frac_of_measured_hbm": gbs / hbm,
                    "sweep_pair_gbs_marginal": mgbs, "sweep_pair_frac_of_measured_hbm": mgbs / hbm,
                    "sweep_pair_us": pair_us, "half_sweep_us": pair_us / 2}
        if prec != 1:
            # FP64 work per cell update: 7 FMA residual + reference divide (or
            # 3 more FMA/MUL of the division-free form)
            out[key]["cell_updates_per_s"] = cells / (pair_us * 1e-6)
    s.close()
    return out


def alu_rates(local):
    import ctypes as C
    from biocfd._lib import check, load
    from biocfd.solver import Solver  # noqa: F401  (initialises the library on the device)
    L = load()
    check(L.bcfd_init(local), "init")
    v = (C.c_double * 3)()
    check(L.bcfd_measure_alu_rates(v), "measure_alu_rates")
    return {"fp64_fma_gflops": v[0], "fp64_div_gops": v[1], "fp32_fma_gflops": v[2],
            "how": "independent FMA / divide chains on every SM (8 CTAs x 256 threads per SM), best of 3 "
                   "CUDA-event timings, no clock changes"}


def twelve_block(torch, local, steps=5, warmup=3, fp64_steps=1, moving=False):
    """Twelve uneven blocks (coarse 320x224x224 + 11 fine blocks, 20.0M cells,
    plate): mixed path batched and per block, plain FP64 to the same residual."""
    from biocfd import synth
    case = synth.twelve_block(n_steps=steps + warmup + 2, moving=moving)
    ncells = sum(b.nx * b.ny * b.nz for b in case.blocks)
    body = case.blocks[1]
    out = {"workload": f"12 blocks: coarse 320x224x224 over 10x7x7 + 11 fine blocks at ratio 2 "
                       f"({body.nx}x{body.ny}x{body.nz} with a plate 0.5x0.125x0.0125, 2x128x64x64, 2x96x64x64, "
                       f"2x64x48x48, 2x48^3, 2x32^3), {ncells / 1e6:.1f}M cells, Re 500" +
                       (", plate heaving 0.5 sin(2 pi 0.25 t) and pitching 30 deg sin(2 pi 0.25 t + 90 deg), "
                        "Search every step" if moving else ", stationary plate") + ", graph replay"}
    arms = (("mixed_batched", 1, True, steps), ("mixed_per_block", 1, False, steps),
            ("fp64_fast_batched", 3, True, fp64_steps))
    for key, prec, batching, n in arms:
        if n <= 0:
            continue
        from biocfd.solver import Solver
        s = Solver(case if prec == 1 else synth.with_mixed_omega(case), device=local)
        s.set_batching(batching)
        s.setup()
        s.set_warm_start(WARM_START)
        s.autotune()
        for _ in range(warmup if prec == 1 else 1):
            s.run(1, precision=prec, div_tol=DIV_TOL, use_graph=1)
        ts, nl = timed_steps(s, torch, n, prec)
        res, _ = residual_stats(s)
        ms = statistics.mean(ts)
        out[key] = {"ms_per_step": ms, "steps_per_s": 1000.0 / ms, "steps": n, "div_residual": res,
                    "launches_per_step": nl / n, "cell_updates_per_s": ncells * 1000.0 / ms}
        s.close()
    if "fp64_fast_batched" in out:
        out["speedup_mixed_vs_fp64_fast"] = (out["fp64_fast_batched"]["ms_per_step"] /
                                             out["mixed_batched"]["ms_per_step"])
    out["speedup_batched_vs_per_block"] = (out["mixed_per_block"]["ms_per_step"] /
                                           out["mixed_batched"]["ms_per_step"])
    return out


def adjoint_bench(torch, local, steps=4, every=2):
    """Discrete adjoint of whole FP64 steps on the 64^3 sphere block (D = 0.25,
    Re 100): time per step of forward + checkpointed reverse pass for the
    objective "time-averaged drag + lift coefficients"."""
    from biocfd import synth
    from biocfd.adjoint import adjoint_run
    from biocfd.solver import Solver
    case = synth.sphere_single_block(n=64, n_steps=steps + 2)
    out = {"workload": f"64^3 sphere block (D=0.25, Re 100), {steps} FP64 steps, checkpoint every {every}, "
                       "objective mean of drag + lift coefficients", "adj_tol": 1e-13}
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
    return out


def adjoint_flapping(torch, steps=200, every=20, fd=(), size="full", epsi=1e-12):
    """Discrete adjoint through the flapping plate of a coarse 128x96x96 +
    fine 128^3 pair (Re 300, heave 0.5 sin(2 pi 0.25 t), pitch 30 deg
    sin(2 pi 0.25 t + 90 deg), a thin-surface plate): `steps` FP64 drop-in
    steps checkpointed every `every`, J = time-averaged drag + lift
    coefficients, its gradient with respect to the five motion parameters and
    the inflow velocity; optional central differences ("name:rel" items of
    `fd`).  The forward solves relax with the mixed path's default factor and stop at the
    reference's increment test with epsi (1e-12 by default, so that the
    differences see the discretisation, not the stopping noise)."""
    import dataclasses
    from biocfd import synth
    from biocfd.adjoint import MOTION_PARAMS, adjoint_run_motion
    from biocfd.solver import Solver
    base = synth.with_mixed_omega(synth.replace(synth.flapping_plate_pair(n_steps=steps, size=size), epsi=epsi,
                                                pc_ita_max=200000))
    seed = (1.0, 1.0, 1.0, 1.0)

    def make(**mv):
        blocks = list(base.blocks)
        own = {k: v for k, v in mv.items() if k in ("yamp", "a0_deg", "bfreq")}
        inputs = {k: v for k, v in mv.items() if k in ("phase_deg", "freq")}
        if own:
            blocks[1] = dataclasses.replace(blocks[1], motion=dataclasses.replace(blocks[1].motion, **own))
        kw = {"uc": mv["uc"]} if "uc" in mv else {}
        return synth.replace(base, blocks=blocks, motion=dataclasses.replace(base.motion, **inputs), **kw)

    def run(case, gradient):
        s = Solver(case)
        s.setup()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = adjoint_run_motion(s, {}, steps, every=every, block=1, gradient=gradient, stress_seed=seed,
                               mu_f=1.0 / case.re, rho_f=1.0, adj_tol=1e-12)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
        counts = s.counts(s.handles[1])
        s.close()
        return r, secs, counts

    (J, duc, g), secs, counts = run(base, True)
    mo, mi = base.blocks[1].motion, base.motion
    p0 = {"yamp": mo.yamp, "a0_deg": mo.a0_deg, "phase_deg": mi.phase_deg, "freq": mi.freq, "bfreq": mo.bfreq,
          "uc": base.uc}
    cells = sum(b.nx * b.ny * b.nz for b in base.blocks)
    out = {"workload": f"flapping plate 0.5x0.125x0.0125 (surface 51, thin-surface cells), coarse "
                       f"{base.blocks[0].nx}x{base.blocks[0].ny}x{base.blocks[0].nz} + fine "
                       f"{base.blocks[1].nx}x{base.blocks[1].ny}x{base.blocks[1].nz} ({cells / 1e6:.2f}M cells), "
                       f"Re 300, {steps} FP64 steps, checkpoint every {every}, J = mean of drag + lift coefficients",
           "epsi": epsi, "adj_tol": 1e-12, "J": J, "dJ_duc": duc, "dJ_dmotion": g["motion"],
           "seconds_forward_and_reverse": secs, "ms_per_step_forward_and_reverse": 1000.0 * secs / steps,
           "ts_cells_at_end": counts["TSCellCount"], "ib_cells_at_end": counts["ibCellCount"],
           "motion_params": p0, "fd": []}
    for item in fd:
        name, rel = item.split(":")
        h = float(rel) * abs(p0[name])
        jp, sp, _ = run(make(**{name: p0[name] + h}), False)
        jm, sm, _ = run(make(**{name: p0[name] - h}), False)
        fdv = (jp - jm) / (2 * h)
        adj = duc if name == "uc" else g["motion"][name]
        out["fd"].append({"param": name, "rel_step": float(rel), "fd": fdv, "adjoint": adj, "J_plus": jp,
                          "J_minus": jm, "rel_diff": abs(fdv - adj) / max(abs(fdv), 1e-300)})
        out["ms_per_step_forward_only"] = 500.0 * (sp + sm) / steps
        print(json.dumps(out["fd"][-1]), flush=True)
    return out


def tandem_long(torch, local, fwd=1000, cmp=100, adj=20, every=5, adj_tol=1e-10):
    """The tandem-plate workload (44.0M cells, both plates heaving and
    pitching, the trailing plate 90 deg behind) over a long horizon:
    (1) the mixed path and the division-free FP64 path (at the mixed path's
    relaxation factor) from the same initial state for `cmp` steps, and the
    mixed path's error in every field and in each plate's drag/lift
    coefficients after them; (2) the mixed path continued to `fwd` steps
    (time per step, residual); (3) from there the discrete adjoint of the next
    `adj` FP64 drop-in steps, checkpointed every `every` steps: J = the leading
    plate's time-averaged drag coefficient (viscous + pressure), its gradient
    with respect to the leading plate's heave and pitch amplitude and heave
    frequency, the shared phase angle and pitch frequency (both plates move
    with them) and the inflow velocity, with the adjoint Poisson solves to
    the residual adj_tol."""
    from biocfd import synth
    from biocfd.adjoint import adjoint_run_motion
    case = synth.with_mixed_omega(synth.tandem_plates(n_steps=fwd + adj + 4, moving=True))
    mu_f = 1.0 / case.re
    out = {"workload": "tandem plates, 44.0M cells: coarse 384x256x256 + two fine 256x192x192, both plates "
                       "heaving 0.125 sin(2 pi 0.25 t) and pitching 15 deg sin(2 pi 0.25 t + 90 deg), trailing "
                       "plate 90 deg behind, Re 1000, Search every step",
           "omega": [b.omega for b in case.blocks]}
    ta = []
    if cmp > 0:
        # one solver at a time (the library holds one set of blocks)
        sb = new_solver(case, local)
        tb, _ = timed_steps(sb, torch, cmp, 3)
        snap_b = ([sb.fields(g) for g in sb.handles], [sb.stress(g, mu_f).tolist() for g in sb.handles[1:]])
        res_b, _ = residual_stats(sb)
        sb.close()
    sa = new_solver(case, local)
    if cmp > 0:
        ta, _ = timed_steps(sa, torch, cmp, 1)
        snap_a = ([sa.fields(g) for g in sa.handles], [sa.stress(g, mu_f).tolist() for g in sa.handles[1:]])
        err, coef = field_errors(snap_a[0], snap_b[0], snap_a[1], snap_b[1])
        out["mixed_vs_fp64"] = {"after_steps": cmp, "field_rel_l2": err, "coef_rel": coef,
                                "coefficients": "per plate: viscous drag, pressure drag, viscous lift, pressure lift",
                                "mixed_ms_per_step": statistics.mean(ta), "fp64_ms_per_step": statistics.mean(tb),
                                "fp64_div_residual": res_b,
                                "fp64": "FP64 momentum + division-free FP64 SOR to the residual 1e-6"}
        del snap_b
    tc, _ = timed_steps(sa, torch, fwd - cmp, 1)
    res_a, pairs_a = residual_stats(sa)
    out["forward"] = {"steps": fwd, "ms_per_step_last": statistics.mean(tc[-50:]),
                      "ms_per_step_all": statistics.mean(ta + tc), "seconds": (sum(ta) + sum(tc)) / 1000.0,
                      "div_residual_last_step": res_a, "sweep_pairs_last_step": pairs_a,
                      "leading_plate_coefficients": sa.stress(sa.handles[1], mu_f).tolist()}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J, duc, g = adjoint_run_motion(sa, {}, adj, every=every, block=1, stress_seed=(1.0, 1.0, 0.0, 0.0), mu_f=mu_f,
                                   rho_f=1.0, adj_tol=adj_tol)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    out["adjoint"] = {"steps": adj, "every": every, "adj_tol": adj_tol, "J": J, "dJ_duc": duc,
                      "dJ_dmotion": g["motion"], "seconds_forward_and_reverse": secs,
                      "s_per_step_forward_and_reverse": secs / adj,
                      "objective": "mean over the adjoint steps of the leading plate's viscous + pressure drag "
                                   "coefficients (FP64 drop-in steps from the mixed path's state)"}
    sa.close()
    return out


def profile_run(args):
    """A short run for profiler captures: the chosen workload set up without
    the autotuner (with `--profile-tune`, the shapes it picks on the tandem
    plates, set directly), then `--profile-steps` eagerly issued steps of the mixed
    path (one kernel launch per phase and block, as a replayed graph holds
    them); prints the per-step time and the phase split of the last step."""
    import torch
    from biocfd import synth
    from biocfd._lib import check
    torch.cuda.set_device(0)
    if args.profile_case == "sweeps":
        # FP64 sweeps of one body-free 384x256x256 block (25.2M cells): one
        # launch of 8 sweep pairs with the reference's arithmetic, then one
        # division-free, no autotuner
        case = synth.uniform_block((384, 256, 256), noise=True)
        s = new_solver(case, 0, tune=False)
        g = s.handles[0]
        check(s.L.bcfd_cellcount_solid(g), "cellcount_solid")
        check(s.L.bcfd_compute_div(g), "compute_div")
        out = {}
        for key, prec in (("fp64_reference_sweeps", 0), ("fp64_division_free", 2)):
            s.profile_begin()
            check(s.L.bcfd_block_sor_sweeps(g, 8, prec), "sor_sweeps")
            out[key] = s.profile_end()
        print(json.dumps({"profile_case": "sweeps", "sweep_pairs": 8, "solve_log": out}), flush=True)
        s.close()
        return
    if args.profile_case == "zmarch":
        # FP32 sweeps of one body-free 256x192x192 block (9.4M cells, ~1.5 GB
        # on the device): one correction of 8 sweep pairs with the tiled
        # sweeps (variant 3), then one with the z-marching TMA sweeps (5)
        case = synth.uniform_block((256, 192, 192), noise=True)
        s = new_solver(case, 0, tune=False)
        g = s.handles[0]
        check(s.L.bcfd_cellcount_solid(g), "cellcount_solid")
        check(s.L.bcfd_compute_div(g), "compute_div")
        out = {}
        for key, variant in (("tiled_neighbour_sync", 3), ("zmarch_tma", 5)):
            s.set_mixed_params(variant=variant, block=g)
            s.profile_begin()
            check(s.L.bcfd_block_sor_sweeps(g, 8, 1), "sor_sweeps")
            out[key] = s.profile_end()
        print(json.dumps({"profile_case": "zmarch", "sweep_pairs": 8, "solve_log": out}), flush=True)
        s.close()
        return
    if args.profile_case == "tandem":
        case = synth.tandem_plates(n_steps=args.profile_steps + 2, moving=True)
    else:  # one 256x192x192 block with a plate: the fine-block size, ~1 GB on the device
        case = synth.plate_block(n=(256, 192, 192), n_steps=args.profile_steps + 2)
    s = new_solver(case, 0, tune=False)
    if args.profile_tune:
        # the launch shapes the autotuner picks on the tandem plates, set
        # directly (timings under a profiler would mislead the autotuner):
        # every block's FP32 correction with neighbour-synchronised tiles and
        # its FP64 solve with grid-synchronised tiles, each in launches of its own
        for q, g in enumerate(s.handles):
            s.set_mixed_params(variant=3, block=g)
            s.set_solve_launch(512, 0, 1, block=q)
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    ts = []
    for q in range(args.profile_steps):
        last = q == args.profile_steps - 1
        if last:
            s.profile_begin()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.run(1, precision=1, div_tol=DIV_TOL)
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1))
        if last:
            prof = s.profile_end()
    print(json.dumps({"profile_case": args.profile_case, "ms_per_step": ts, "phases_ms": s.profile_phases(),
                      "kernel_launches_last_step": prof["kernel_launches"],
                      "solve_log_last_step": {k: prof[k] for k in ("sor_launches", "sor_ms", "sor_bytes",
                                                                   "sor_sweeps")},
                      "counts": [s.counts(g) for g in s.handles]}), flush=True)
    s.close()


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    hbm, peak_kind = peaks()
    t_start = time.perf_counter()
    h = headline(args, torch, local, world)
    mixed = h["mixed"]
    fast = h.get("fp64_fast")
    line = {
        "metric": METRIC,
        "value": world * mixed["steps_per_s"],
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": mixed["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 sweeps + f64 defect correction",
        "data": "synthetic (seeded, numpy default_rng 20261203)",
        "config": {"workload": WORKLOAD, "blocks": "384x256x256 + 2 x 256x192x192",
                   "parallelism": f"replicas x{world}",
                   "solve_start": ("warm: every residual-target solve (mixed and FP64 arms alike) starts from "
                                   "the previous step's correction at its fluid cells" if WARM_START else
                                   "zero, as the reference"),
                   "l2": "not flushed: working set ~5 GB, far above the 129 MB L2",
                   "timed": "per-step CUDA events on the library stream",
                   "launch": "each step one replay of the captured step CUDA graph (each step's kinematics "
                             "staged on the host before its replay)"},
        "e2e": h["e2e"],
        "gpu_launches": h["gpu_launches"],
        "roofline": h["roofline"],
        "clocks": h["clocks"],
        "mixed": mixed,
        "phases": h["phases"],
        "cell_updates_per_s": world * mixed["cell_updates_per_s"],
    }
    for key in ("mixed_zero_start", "fp64_fast", "fp64", "fp64_input_omega", "fp64_dropin"):
        if key in h:
            line[key] = h[key]
    if fast:
        line["speedup_vs_fp64"] = fast["ms_per_step"] / mixed["ms_per_step"]
    if not args.no_extras:
        line["alu_rates"] = alu_rates(local)
        line["sweep_roofline"] = sweep_roofline(torch, local, hbm)
        line["two_block"] = two_block(torch, local, steps=10, warmup=3)
        line["twelve_block_moving"] = twelve_block(torch, local, moving=True)
        line["adjoint"] = adjoint_bench(torch, local)
    if rank == 0 and not args.no_cpu_baseline:
        from biocfd import synth
        r = cpu_reference_sample(synth.tandem_plates(n_steps=2, moving=True), REFERENCE_SWEEP_PAIRS)
        line["cpu_baseline"] = {"value": r["steps_per_s"], "unit": "steps/s", "cores": r["threads"],
                                "kind": "port", "sample": r["sample"]}
    line["bench_wall_s"] = time.perf_counter() - t_start
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=1, help="timed steps of each FP64 arm")
    ap.add_argument("--fp64-input-omega", action="store_true",
                    help="also run the plain FP64 arm with the input omega 1.7 (~16 s per step)")
    ap.add_argument("--dropin-steps", type=int, default=0,
                    help="steps of the drop-in FP64 path (reference stop test) on the headline workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the ALU rates, sweep roofline, two-block, twelve-block and adjoint keys")
    ap.add_argument("--sweep-only", default="",
                    help="nx,ny,nz[,fp32_pairs[,fp64_pairs]]: only the Poisson sweep measurement on that block")
    ap.add_argument("--twelve-only", action="store_true", help="only the twelve-block measurement")
    ap.add_argument("--adjoint-only", action="store_true", help="only the adjoint timing")
    ap.add_argument("--adjoint-flapping", default="",
                    help="STEPS[,EVERY[,name:rel;name:rel...]]: only the moving-plate adjoint on the coarse "
                         "128x96x96 + fine 128^3 pair, with optional central differences")
    ap.add_argument("--tandem-long", default="",
                    help="FWD,CMP,ADJ[,EVERY]: only the long tandem-plate run: mixed vs FP64 after CMP steps, FWD "
                         "mixed steps, then the adjoint of ADJ FP64 steps")
    ap.add_argument("--alu-only", action="store_true", help="only the arithmetic-rate measurement")
    ap.add_argument("--zero-start", action="store_true",
                    help="start every residual-target solve from pc = 0 (the reference's start)")
    ap.add_argument("--zero-start-steps", type=int, default=5,
                    help="timed steps of the flagship with zero-started solves, beside the warm-started value")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiler mode: set up without the autotuner and run this many eager mixed steps")
    ap.add_argument("--profile-case", default="tandem", choices=["tandem", "block256", "sweeps", "zmarch"])
    ap.add_argument("--profile-tune", action="store_true",
                    help="profiling run: the launch shapes the autotuner picks on the tandem plates, set directly")
    args = ap.parse_args()
    global WARM_START
    WARM_START = not args.zero_start
    if args.warmup < 3:
        args.warmup = 3
    if args.sweep_only:
        import torch
        v = [int(x) for x in args.sweep_only.split(",")]
        hbm, _ = peaks()
        print(json.dumps(sweep_roofline(torch, 0, hbm, v[:3], v[3] if len(v) > 3 else 40,
                                        v[4] if len(v) > 4 else 8)), flush=True)
        return
    if args.twelve_only:
        import torch
        print(json.dumps(twelve_block(torch, 0, args.steps, args.warmup)), flush=True)
        print(json.dumps(twelve_block(torch, 0, args.steps, args.warmup, moving=True)), flush=True)
        return
    if args.adjoint_only:
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(adjoint_bench(torch, 0)), flush=True)
        return
    if args.adjoint_flapping:
        import torch
        torch.cuda.set_device(0)
        v = args.adjoint_flapping.split(",")
        fd = tuple(x for x in v[2].split(";") if x) if len(v) > 2 else ()
        print(json.dumps(adjoint_flapping(torch, int(v[0]), int(v[1]) if len(v) > 1 else 20, fd)), flush=True)
        return
    if args.tandem_long:
        import torch
        torch.cuda.set_device(0)
        v = [int(x) for x in args.tandem_long.split(",")]
        print(json.dumps(tandem_long(torch, 0, v[0], v[1], v[2], v[3] if len(v) > 3 else 5)), flush=True)
        return
    if args.alu_only:
        print(json.dumps(alu_rates(0)), flush=True)
        return
    if args.profile_steps > 0:
        profile_run(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
