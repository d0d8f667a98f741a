#!/usr/bin/env python
"""Benchmark of the GB300 time-stepping engine on the layered 2048x2048 case.

Workload ("layered-grf-2048"): MX = MZ = 2048 with a 20-cell PML
(2088 x 2071 = 4,324,248 cells counting the PML), dx = 1 m, dt = 1e-4 s,
a sandstone half-space over a tight layer at 1024 m, both perturbed by a
10 % Gaussian random field (correlation 20 m), one material per cell,
free surface by stress imaging, 20 Hz Ricker explosive source at 10 m,
512 receivers on row 2; FP32.  Seeded synthetic inputs stand in for the
reference's own model files, which its repository does not contain.

A "step" is one time level of the whole grid (both half-steps, all
boundary rows, receiver sampling).  The metric is cell-updates per second
counting the PML cells.  The fields and per-cell media (~0.6 GB) are larger
than L2, so no flush is needed between timed levels.

Arms:
  default            the CUDA engine (value, e2e through the C ABI, roofline
                     of the dominant kernel, CPU baseline on a sample)
  --impl reference   the CPU restatement of the reference's time loop
                     (OpenMP over rows, all host threads), same workload

Other workloads (--workload): batch (64 shots of uneven sizes, shots/hour
against the same shots one after another, and against the plain FP64
single-shot path), large (16 shots of 8192^2 over one shared medium) and
edge (the learned absorbing edge against the strip alone and the PMLs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "2d-vqsp-fd-sim_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOAD = dict(mx=2048, mz=2048, tpml=20, h=1.0, dt=1e-4, mt2=4000, f0=20.0, n_rec=512, seed=20250)
METRIC = "Gcell-updates/s"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _barrier_max(value: float, ws: int) -> float:
    if ws <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(ws: int) -> None:
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def prepare_inputs(precision: str, mt2: int):
    from fdporo import job
    w = WORKLOAD
    cfg, med = job.layered(mx=w["mx"], mz=w["mz"], nsteps=mt2, tpml=w["tpml"], f0=w["f0"], dt=w["dt"], h=w["h"],
                           n_rec=w["n_rec"], seed=w["seed"], layer_depth=1024.0)
    return job.prepare(cfg, med, precision)


def algorithmic_bytes(inp, s: int, medium: dict, core: dict | None = None, march: dict | None = None) -> dict:
    """Compulsory DRAM bytes per launch of each phase for this workload:
    every wavefield value the phase reads or read-modify-writes, the
    material coefficients of each cell as the engine holds them (one value
    per distinct coefficient plane, or the JM index in table mode), and
    every PML memory variable it updates (read + write).  Damping profiles
    and a material table are small and cache-resident and are not counted.
    With the core rectangles, also the bytes of each core kernel (its cells
    only: no PML memory)."""
    nx, nz, tp = inp.nx, inp.nz, inp.tpml
    cells = nx * nz
    if medium["mode"] == "table":
        med_s = med_v = 4
    else:
        med_s, med_v = medium["planes_stress"] * s, medium["planes_velocity"] * s
    # element counts of the memory variables (ppml.F90:85-112)
    side = lambda w: w * nz
    bottom = lambda h: nx * h
    stress_mem = (side(tp + 2) + side(tp + 1) + 2 * side(tp + 1) + 2 * side(tp + 1)
                  + bottom(tp + 2) + 2 * bottom(tp + 1))
    vel_mem = (4 * side(tp + 3) + 4 * side(tp + 2) + 2 * side(tp + 2) + 2 * side(tp + 2) + 6 * bottom(tp + 1))
    stress = cells * (4 * s + 8 * s + med_s) + 2 * s * stress_mem
    velocity = cells * (4 * s + 8 * s + med_v) + 2 * s * vel_mem + 2 * s * 12 * nx
    out = {"stress": stress, "velocity": velocity, "per_cell_stress": stress / cells,
           "per_cell_velocity": velocity / cells}
    if core:
        x0, x1, z0, z1 = core["stress"]
        ns = max(x1 - x0, 0) * max(z1 - z0, 0)
        if ns and z0 <= inp.lin_z < z1:
            ns -= x1 - x0  # the source row is not a core row
        x0, x1, z0, z1 = core["velocity"]
        nv = max(x1 - x0, 0) * max(z1 - z0, 0)
        out["stress_core"] = ns * (12 * s + med_s)
        out["velocity_core"] = nv * (12 * s + med_v)
        out["core_cells"] = {"stress": ns, "velocity": nv}
    if march:
        # the march kernel: per cell of its region the old velocities and
        # stresses read once, the new velocities written, and the medium of
        # both phases; the new stresses written where it writes them (the
        # frame kernels write the band along its edges)
        x0, x1, z0, z1 = march["region"]
        nf = (x1 - x0) * (z1 - z0)
        x0, x1, z0, z1 = march["stress_writes"]
        nw = (x1 - x0) * (z1 - z0)
        out["march"] = nf * (12 * s + med_s + med_v) + nw * 4 * s
        # the whole level: both phases' bytes less the second reads of the
        # new stresses and the old velocities that the march kernel saves
        out["level"] = stress + velocity - nf * 8 * s
        out["march_cells"] = {"region": nf, "stress_writes": nw}
    return out


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if parts[4 + k].lower().startswith("active"):
                    reasons.add(n)
        busy = sorted(sm)[len(sm) // 2:] if sm else []
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def ncu_traffic(kernel: str) -> float | None:
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return float(d[kernel]["dram_bytes_per_launch_full_size"])
    except Exception:
        return None


def cpu_time_levels(inp, levels: int, warmup: int, threads: int, ascii_io: bool = False) -> tuple[float, int]:
    """Seconds for ``levels`` time levels of the oracle (after ``warmup``),
    and the receiver files opened.  With ``ascii_io`` every level is followed
    by the reference's receiver output (store_seismograms.F90:140-154,
    store_seismograms_pressure.F90:76-83): per receiver an OPEN with
    POSITION='APPEND', one E13.6 line and a CLOSE of each of its two or three
    files, here into a temporary directory."""
    import tempfile

    from oracle.oracle import make_oracle
    o = make_oracle(inp, threads=threads)
    if warmup:
        o.time_loop(1, warmup)
    opened = 0
    with tempfile.TemporaryDirectory() as d:
        t = time.perf_counter()
        if ascii_io:
            opened = o.time_loop_ascii(warmup + 1, warmup + levels, d)
        else:
            o.time_loop(warmup + 1, warmup + levels)
        el = time.perf_counter() - t
    o.close()
    return el, opened


def cpu_baseline_sample(inp, threads: int, seconds: float) -> dict:
    """The oracle on a bounded sample of the workload: kernel-only levels from
    rest (about ``seconds`` of work), and fewer levels with the reference's
    per-level ASCII receiver output."""
    t1, _ = cpu_time_levels(inp, 2, 0, threads)
    lv = int(max(2, min(200, seconds / max(t1 / 2, 1e-6))))
    el, _ = cpu_time_levels(inp, lv, 0, threads)
    lv_io = max(2, lv // 4)
    el_io, opened = cpu_time_levels(inp, lv_io, 0, threads, ascii_io=True)
    return {"value": inp.cells * lv / el / 1e9, "unit": METRIC, "cores": threads, "kind": "port",
            "sample": f"{lv} full-grid time levels from rest ({el:.1f} s; C++ restatement of the reference "
                      "time loop, OpenMP over rows)",
            "with_ascii_io": {"value": inp.cells * lv_io / el_io / 1e9, "unit": METRIC, "levels": lv_io,
                              "seconds": el_io, "files_per_level": opened // lv_io,
                              "pattern": "after each level, per receiver OPEN(POSITION='APPEND')/WRITE one "
                                         "E13.6 line/CLOSE of REC_UW_<j>.asc, REC_Q_<j>.asc (KEY_TLQ) and "
                                         "REC_STRESS_<j>.asc (KEY_TLP), as store_seismograms(_pressure).F90"}}


def run_reference(args) -> None:
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    inp = prepare_inputs(args.precision, max(WORKLOAD["mt2"], args.warmup + args.steps))
    el, _ = cpu_time_levels(inp, args.steps, args.warmup, threads)
    value = inp.cells * args.steps / el / 1e9
    lv_io = max(2, args.steps // 4)
    el_io, opened = cpu_time_levels(inp, lv_io, args.warmup, threads, ascii_io=True)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "f32" else "f64",
        "data": "synthetic (seeded layered medium with Gaussian random field)",
        "config": {"workload": "layered-grf-2048", "cells": inp.cells, "mx": WORKLOAD["mx"], "mz": WORKLOAD["mz"],
                   "tpml": WORKLOAD["tpml"], "levels_per_shot": WORKLOAD["mt2"], "media": "per-cell"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full-grid time levels after {args.warmup} warm-up levels "
                                   "(C++ restatement of the reference time loop, OpenMP over rows)",
                         "with_ascii_io": {"value": inp.cells * lv_io / el_io / 1e9, "unit": METRIC,
                                           "levels": lv_io, "files_per_level": opened // lv_io,
                                           "pattern": "per level and receiver OPEN(APPEND)/WRITE/CLOSE of its "
                                                      "seismogram files, as store_seismograms(_pressure).F90"}},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args) -> None:
    import torch
    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = local if torch.cuda.is_available() else 0
    torch.cuda.set_device(dev)
    from fdporo import job

    prof_levels = 50
    mt2 = max(WORKLOAD["mt2"], args.warmup + args.steps + prof_levels)
    inp = prepare_inputs(args.precision, mt2)
    s = 8 if args.precision == "f64" else 4
    eng = job.make_engine(inp, device=dev)
    ext = torch.cuda.ExternalStream(eng.stream(), device=dev)

    # ---- the CUDA graphs of the warm-up and of a run of args.steps levels
    # are captured here, before the clock starts (fdp_run replays them)
    eng.prepare_run(args.warmup)
    eng.prepare_run(args.steps)
    eng.synchronize()
    # ---- timed region, right after the warm-up levels (which run once the
    # clock sampler is up, so that the GPU goes from them straight into the
    # timed levels instead of from an idle pause)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        _barrier(ws)
        eng.time_loop(1, args.warmup)
        n0 = eng.kernel_launches()
        torch.cuda.synchronize()
        e0.record(ext)
        eng.time_loop(args.warmup + 1, args.warmup + args.steps)
        e1.record(ext)
        e1.synchronize()
        torch.cuda.synchronize()
    launches = eng.kernel_launches() - n0
    ms = e0.elapsed_time(e1)
    ms_max = _barrier_max(ms, ws)
    value = inp.cells * args.steps * ws / (ms_max / 1e3) / 1e9

    # ---- per-kernel device time (separate launches between events)
    lo = args.warmup + args.steps + 1
    prof = eng.profile(lo, lo + prof_levels - 1)
    medium = eng.medium_info()
    core = eng.core_info()
    march = eng.march_info()
    alg = algorithmic_bytes(inp, s, medium, core, march)
    phases = ("stress", "velocity", "edge")
    shares = {k: prof[k][0] / max(sum(prof[q][0] for q in phases), 1e-30) for k in phases}
    peak, peak_kind = measured_peak_gbs()
    if march:
        # one pass per level over the deep interior (the march kernel) beside
        # the frame kernels: the level's time is entry "stress" of the profile
        kern = "march"
        avg_ms = prof["stress_core"][0] / prof["stress_core"][1]
        level_ms = prof["stress"][0] / prof["stress"][1]
        phase_gbs = {"level": alg["level"] / (level_ms / 1e3) / 1e9}
    else:
        # the dominant kernel: that of the longer phase -- its core kernel
        # when the phase runs as frame and core kernels on two streams, else
        # the phase's one kernel
        phase = max(("stress", "velocity"), key=lambda k: prof[k][0])
        kern = f"{phase}_core" if prof[f"{phase}_core"][1] > 0 else phase
        avg_ms = prof[kern][0] / prof[kern][1]
        phase_gbs = {k: alg[k] / (prof[k][0] / prof[k][1] / 1e3) / 1e9 for k in ("stress", "velocity")}
    achieved = alg[kern] / (avg_ms / 1e3) / 1e9
    level_bytes = alg["level"] if march else alg["stress"] + alg["velocity"]
    eng.close()

    # ---- end to end through the C ABI: one whole shot (create, upload, run, download)
    e2e = None
    if not args.no_e2e:
        from fdporo.engine import Engine
        torch.cuda.synchronize()
        t = time.perf_counter()
        e = Engine(inp.mx, inp.mz, inp.tpml, inp.lin_x, inp.lin_z, inp.h, inp.dt, precision=args.precision,
                   stress_imaging=inp.stress_imaging, device=dev)
        t_create = time.perf_counter()
        e.set_medium(inp.jm, inp.table)
        t_medium = time.perf_counter()
        e.set_pml(inp.profiles)
        e.set_bottom_nr(inp.ab)
        e.set_source(inp.sourtf)
        e.set_receivers(inp.irecx, inp.lrecx, inp.irecz, inp.lrecz, inp.rec_flags)
        t_set = time.perf_counter()
        e.time_loop(1, WORKLOAD["mt2"])
        e.synchronize()
        t_run = time.perf_counter()
        rec = e.receivers(1, WORKLOAD["mt2"])
        el = time.perf_counter() - t
        breakdown = {"create_s": t_create - t, "set_medium_s": t_medium - t_create,
                     "set_pml_bottom_source_receivers_s": t_set - t_medium, "levels_s": t_run - t_set,
                     "receivers_s": t + el - t_run}
        e.close()
        h2d = (inp.jm.nbytes + inp.table.nbytes + sum(p.nbytes for p in inp.profiles) + inp.ab.nbytes
               + inp.sourtf[: WORKLOAD["mt2"]].nbytes + 16 * len(inp.irecx))
        e2e = {"value": inp.cells * WORKLOAD["mt2"] * ws / _barrier_max(el, ws) / 1e9, "unit": METRIC,
               "h2d_bytes_per_step": h2d // WORKLOAD["mt2"], "d2h_bytes_per_step": rec.nbytes // WORKLOAD["mt2"],
               "shot_seconds": el, "shots_per_hour": 3600.0 / el, "breakdown": breakdown,
               "scope": f"one whole shot of {WORKLOAD['mt2']} levels: fdp_create, fdp_set_* from host buffers, "
                        "fdp_run, fdp_get_receivers"}

    # ---- seismogram error of this precision against the FP64 engine, whose
    # every value the parity tests pin bit for bit to the FP64 oracle
    accuracy = None
    if e2e is not None and args.precision == "f32" and not args.no_accuracy:
        inp64 = prepare_inputs("f64", WORKLOAD["mt2"])
        e64 = job.make_engine(inp64, device=dev)
        e64.time_loop(1, WORKLOAD["mt2"])
        rec64 = e64.receivers(1, WORKLOAD["mt2"])
        e64.close()
        cols = [0, 1, 8, 9]  # SSU, SSW (u, -w) and SSP, SST (p, -txx)
        ref = rec64[:, :, cols]
        diff = rec.astype(np.float64)[:, :, cols] - ref
        accuracy = {"seismogram_rel_l2": float(np.linalg.norm(diff) / np.linalg.norm(ref)),
                    "against": "FP64 engine over the same whole shot (u, -w, p, -txx at all receivers and levels)",
                    "target": 1e-3}

    # ---- batched shots against the same shots one by one (rank 0, N = 1)
    batch = None
    if rank == 0 and ws == 1 and not args.no_batch:
        batch = batch_leg(dev)

    # ---- CPU baseline on a bounded sample (rank 0, N = 1 only)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline_sample(inp, os.cpu_count() or 1, args.cpu_seconds)

    if rank != 0:
        return
    step_s = ms_max / 1e3 / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if args.precision == "f32" else "f64",
        "data": "synthetic (seeded layered medium with Gaussian random field)",
        "config": {"workload": "layered-grf-2048", "cells": inp.cells, "mx": WORKLOAD["mx"], "mz": WORKLOAD["mz"],
                   "tpml": WORKLOAD["tpml"], "media": "per-cell", "levels_per_shot": WORKLOAD["mt2"],
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"shot replicas x{ws}",
                   "graphs": "the timed levels replay CUDA graphs captured before the timed region",
                   "shots_per_hour_device": 3600.0 / (step_s * WORKLOAD["mt2"])},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": kern, "achieved": achieved, "peak": peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": ncu_traffic(kern),
                     "alg_bytes_per_launch": alg[kern], "avg_launch_ms": avg_ms,
                     "alg_bytes_per_cell": {"stress": alg["per_cell_stress"], "velocity": alg["per_cell_velocity"]},
                     "kernel_ms": {k: prof[k][0] / max(prof[k][1], 1) for k in prof},
                     "phase_gbs": phase_gbs, "phase_frac": {k: v / peak for k, v in phase_gbs.items()},
                     # the whole level's compulsory bytes over the timed level
                     # (the timed region's graphs, frame and core side by side)
                     "level_gbs_timed": level_bytes / (ms_max / args.steps / 1e3) / 1e9,
                     "level_frac_timed": level_bytes / (ms_max / args.steps / 1e3) / 1e9 / peak,
                     "core_cells": alg.get("core_cells"), "march": march, "march_cells": alg.get("march_cells"),
                     "medium": medium, "phase_share": shares},
        "e2e": e2e,
        "accuracy": accuracy,
        "batch": batch,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


BATCH = dict(shots=64, mt2=3000, seed=20251)


def _prepare_batch_shot(item, precision: str = "f32"):
    """Prepared inputs of one shot of the batched workload (runs in a worker
    process; the result is uploaded by the parent)."""
    from fdporo import job
    seed, kw = item
    cfg, med = job.batch_shot(seed, **kw)
    return job.prepare(cfg, med, precision)


def _prepare_batch_shot_f64(item):
    return _prepare_batch_shot(item, "f64")


def plain_fp64_comparison(shots, dev: int, levels: int = 10) -> dict:
    """The plain single-shot path in the reference's working precision
    (REAL(8)): every shot of the batch alone through fdp_run in FP64, timed
    over `levels` levels each; and the FP32 seismogram error against FP64
    over the whole run of the smallest shot."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch
    from fdporo import job
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms, cells, small = 0.0, [], None
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as pool:
        for item, inp in zip(shots, pool.map(_prepare_batch_shot_f64, shots)):
            e = job.make_engine(inp, device=dev)
            e.time_loop(1, 3)
            e.prepare_run(levels)
            s = torch.cuda.ExternalStream(e.stream(), device=dev)
            e0.record(s)
            e.time_loop(4, 3 + levels)
            e1.record(s)
            e1.synchronize()
            ms += e0.elapsed_time(e1) / levels
            e.close()
            cells.append(inp.cells)
            if small is None or inp.cells < small[1]:
                small = (item, inp.cells)
    # FP32 against FP64 over a whole run of the smallest shot
    item = small[0]
    recs = []
    for prec in ("f32", "f64"):
        inp = _prepare_batch_shot(item, prec)
        e = job.make_engine(inp, device=dev)
        e.time_loop(1, inp.mt2)
        recs.append(e.receivers(1, inp.mt2)[:, :, [0, 1, 8, 9]].astype(np.float64))
        e.close()
    err = float(np.linalg.norm(recs[0] - recs[1]) / max(np.linalg.norm(recs[1]), 1e-300))
    return {"ms_per_level": ms, "levels_timed_per_shot": levels, "cells_per_level": sum(cells),
            "fp32_seismogram_rel_l2_vs_fp64": err, "error_shot_cells": small[1]}


def batch_leg(dev: int, levels: int = 32) -> dict:
    """The batched-shots comparison, bounded, for the default run: the 64
    shots of the batch workload (sides 512..2048, per-shot media, 20-cell
    PML, FP32) advanced together by fdp_batch over `levels` timed levels
    after the batch tuned its shape on 50 levels, against the same shots one
    after another through fdp_run in FP32 and in FP64 (the reference's
    working precision), with the FP32 seismogram error against FP64 over
    the whole run of the smallest shot.  shots/hour are for BATCH['mt2']
    levels per shot."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch
    from fdporo import job
    from fdporo.engine import Batch
    shots = job.batch_shots(BATCH["shots"], nsteps=BATCH["mt2"], seed=BATCH["seed"])
    engines, cells = [], []
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as pool:
        for inp in pool.map(_prepare_batch_shot, shots):
            engines.append(job.make_engine(inp, device=dev))
            cells.append(inp.cells)
    setup_s = time.perf_counter() - t0
    total = sum(cells)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    W = 50
    b = Batch(engines)
    ext = torch.cuda.ExternalStream(b.stream(), device=dev)
    b.time_loop(1, W)
    b.synchronize()
    e0.record(ext)
    b.time_loop(W + 1, W + levels)
    e1.record(ext)
    e1.synchronize()
    ms_batch = e0.elapsed_time(e1) / levels
    shape = b.shape()
    b.close()
    # the same shots one after another (FP32), each replaying its own graphs
    lo = W + levels + 1
    ms_seq = 0.0
    for e in engines:
        e.prepare_run(levels)
        e.time_loop(lo, lo + 2)
        s = torch.cuda.ExternalStream(e.stream(), device=dev)
        e0.record(s)
        e.time_loop(lo + 3, lo + 2 + levels)
        e1.record(s)
        e1.synchronize()
        ms_seq += e0.elapsed_time(e1) / levels
        e.close()
    per_hour = lambda ms: BATCH["shots"] * 3600.0 / (BATCH["mt2"] * ms / 1e3)
    fp64 = plain_fp64_comparison(shots, dev)
    return {"shots": BATCH["shots"], "cells_per_level": total, "levels_timed": levels, "setup_s": setup_s,
            "tile_shape": {"units_per_item": shape[0], "waves": shape[1]},
            "batch_fp32": {"ms_per_level": ms_batch, "shots_per_hour": per_hour(ms_batch),
                           "gcell_updates_per_s": total / (ms_batch / 1e3) / 1e9},
            "sequential_fp32": {"ms_per_level": ms_seq, "shots_per_hour": per_hour(ms_seq)},
            "sequential_fp64": {"ms_per_level": fp64["ms_per_level"], "shots_per_hour": per_hour(fp64["ms_per_level"]),
                                "levels_timed_per_shot": fp64["levels_timed_per_shot"]},
            "batch_vs_sequential_fp32": ms_seq / ms_batch,
            "batch_fp32_vs_sequential_fp64": fp64["ms_per_level"] / ms_batch,
            "fp32_seismogram_rel_l2_vs_fp64": fp64["fp32_seismogram_rel_l2_vs_fp64"],
            "note": "the factor against the FP64 single-shot path is FP32 against FP64 on HBM-bound kernels; "
                    "batching itself is batch_vs_sequential_fp32"}


def run_batch(args) -> None:
    """Batched workload: BATCH['shots'] shots with grid sides drawn from
    512..2048 (multiples of 32), per-shot layered random media, sources in
    the upper quarter, 20-cell PML, FP32, advanced together by fdp_batch
    (one launch per phase per level, tile shape tuned on the warm-up
    levels), against the same shots run one after another with fdp_run."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch
    from fdporo import job
    from fdporo.engine import Batch
    ws, rank, local = _dist()
    dev = local if torch.cuda.is_available() else 0
    shots = job.batch_shots(args.shots, nsteps=BATCH["mt2"], seed=BATCH["seed"])
    engines, cells = [], []
    t0 = time.perf_counter()
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as pool:
        for inp in pool.map(_prepare_batch_shot, shots):
            engines.append(job.make_engine(inp, device=dev))
            cells.append(inp.cells)
    setup_s = time.perf_counter() - t0
    total = sum(cells)
    # the batch tunes its shape on its first 50 levels (9 queue shapes x 2,
    # then one 32-level graph of the shots mode)
    K, W = args.steps, max(args.warmup, 50)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    b = Batch(engines)
    ext = torch.cuda.ExternalStream(b.stream(), device=dev)
    b.time_loop(1, W)
    b.synchronize()
    launches0 = b.kernel_launches()
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        e0.record(ext)
        b.time_loop(W + 1, W + K)
        e1.record(ext)
        e1.synchronize()
    ms_batch = e0.elapsed_time(e1) / K
    launches = b.kernel_launches() - launches0
    shape = b.shape()
    b.synchronize()
    b.close()

    # the same shots one after another, each with its own stream and graphs
    lo = W + K + 1
    for e in engines:
        e.time_loop(lo, lo + W - 1)
    for e in engines:
        e.synchronize()
    lo += W
    ms_seq = 0.0
    for e in engines:
        e.prepare_run(K)
        s = torch.cuda.ExternalStream(e.stream(), device=dev)
        e0.record(s)
        e.time_loop(lo, lo + K - 1)
        e1.record(s)
        e1.synchronize()
        ms_seq += e0.elapsed_time(e1) / K
    for e in engines:
        e.close()
    per_shot = lambda ms: args.shots * 3600.0 / (BATCH["mt2"] * ms / 1e3)
    fp64 = plain_fp64_comparison(shots, dev)
    # the same shots with a 4-cell PML (the width of the learned edge's
    # strip; on the learned-edge media it absorbs as well as the 20-cell
    # one), batched the same way
    thin = job.batch_shots(args.shots, nsteps=BATCH["mt2"], seed=BATCH["seed"], tpml=4)
    with ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 1), mp_context=mp.get_context("spawn")) as pool:
        engines = [job.make_engine(inp, device=dev) for inp in pool.map(_prepare_batch_shot, thin)]
    b = Batch(engines)
    ext = torch.cuda.ExternalStream(b.stream(), device=dev)
    b.time_loop(1, W)
    b.synchronize()
    e0.record(ext)
    b.time_loop(W + 1, W + K)
    e1.record(ext)
    e1.synchronize()
    ms_thin = e0.elapsed_time(e1) / K
    b.close()
    for e in engines:
        e.close()
    line = {
        "metric": "shots/hour", "value": per_shot(ms_batch), "unit": "shots/hour", "n_gpus": 1, "steps": K,
        "warmup": W, "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded layered media with Gaussian random fields, one per shot)",
        "config": {"workload": f"batch-{args.shots}", "shots": args.shots, "cells_per_level": total,
                   "sides": "512..2048 step 32", "tpml": 20, "levels_per_shot": BATCH["mt2"],
                   "l2": "inputs larger than L2 (no flush)", "setup_s": setup_s},
        "gcell_updates_per_s": total / (ms_batch / 1e3) / 1e9,
        "sequential": {"ms_per_level": ms_seq, "shots_per_hour": per_shot(ms_seq),
                       "gcell_updates_per_s": total / (ms_seq / 1e3) / 1e9},
        "speedup_vs_sequential": ms_seq / ms_batch,
        # the plain single-shot path in the reference's working precision
        "plain_fp64_single_shot": dict(fp64, shots_per_hour=per_shot(fp64["ms_per_level"])),
        "speedup_vs_plain_fp64_single_shot": fp64["ms_per_level"] / ms_batch,
        "batch_4_cell_pml": {"ms_per_level": ms_thin, "shots_per_hour": per_shot(ms_thin),
                             "speedup_vs_20_cell_batch": ms_batch / ms_thin,
                             "speedup_vs_plain_fp64_single_shot": fp64["ms_per_level"] / ms_thin},
        "tile_shape": {"units_per_item": shape[0], "waves": shape[1]},
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


LARGE = dict(shots=16, mx=8192, mz=8192, mt2=10000, seed=20252)


def run_large(args) -> None:
    """Large survey: LARGE['shots'] shots over one 8192^2 layered random
    medium (per-cell, config-2 generator, free surface on top, 20-cell PML
    on the other sides), sources uniform in the upper quarter, FP32.  The
    medium is derived and uploaded once and shared by every shot
    (fdp_share_medium); all field state stays on the device; the shots are
    advanced together by fdp_batch.  Compared with the plain single-shot
    path: the first shot alone through fdp_run."""
    import torch
    from fdporo import job
    from fdporo.engine import Batch
    ws, rank, local = _dist()
    dev = local if torch.cuda.is_available() else 0
    n = args.shots if args.shots != BATCH["shots"] else LARGE["shots"]
    t0 = time.perf_counter()
    cfg, med, pos = job.large_shots(n, mx=LARGE["mx"], mz=LARGE["mz"], nsteps=LARGE["mt2"], seed=LARGE["seed"])
    inp = job.prepare(cfg, med, "f32")
    del med
    t_prep = time.perf_counter() - t0
    free0 = torch.cuda.mem_get_info(dev)[0]
    t0 = time.perf_counter()
    owner = job.make_engine(inp, device=dev)
    engines = [owner] + [job.make_engine(job.with_source(inp, cfg, x, z), device=dev, medium_from=owner)
                         for x, z in pos[1:]]
    t_upload = time.perf_counter() - t0
    used = free0 - torch.cuda.mem_get_info(dev)[0]
    medium = owner.medium_info()
    core = owner.core_info()
    # the planes as the engine pads them: pitch of NX + 8 rounded up to 32, NZ + 4 rows
    pitch = (inp.nx + 8 + 31) // 32 * 32
    plane_bytes = (medium["planes_stress"] + medium["planes_velocity"]) * 4 * pitch * (inp.nz + 4)
    march = owner.march_info()
    ab = algorithmic_bytes(inp, 4, medium, core, march)
    # a level's compulsory bytes: 104 B per cell of a march level's deep
    # interior, both phases' bytes elsewhere
    level_bytes = n * (ab["level"] if march else ab["stress"] + ab["velocity"])
    cells = n * inp.cells
    # the batch tunes its shape on its first 50 levels (9 queue shapes x 2,
    # then one 32-level graph of the shots mode)
    K, W = args.steps, max(args.warmup, 50)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b = Batch(engines)
    ext = torch.cuda.ExternalStream(b.stream(), device=dev)
    b.time_loop(1, W)
    b.synchronize()
    launches0 = b.kernel_launches()
    with ClockSampler(dev) as clk:
        torch.cuda.synchronize()
        e0.record(ext)
        b.time_loop(W + 1, W + K)
        e1.record(ext)
        e1.synchronize()
    ms_batch = e0.elapsed_time(e1) / K
    launches = b.kernel_launches() - launches0
    shape = b.shape()
    b.synchronize()
    b.close()
    for e in engines[1:]:
        e.close()
    # the plain single-shot path: the first shot alone
    lo = W + K + 1
    owner.time_loop(lo, lo + W - 1)
    owner.prepare_run(K)
    owner.synchronize()
    lo += W
    st = torch.cuda.ExternalStream(owner.stream(), device=dev)
    e0.record(st)
    owner.time_loop(lo, lo + K - 1)
    e1.record(st)
    e1.synchronize()
    ms_single = e0.elapsed_time(e1) / K
    owner.close()
    peak, peak_kind = measured_peak_gbs()
    gbs = level_bytes / (ms_batch / 1e3) / 1e9
    shots_h = lambda ms, k: k * 3600.0 / (LARGE["mt2"] * ms / 1e3)
    line = {
        "metric": "Gcell-updates/s", "value": cells / (ms_batch / 1e3) / 1e9, "unit": "Gcell-updates/s",
        "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (one seeded layered medium with a Gaussian random field, shared by every shot)",
        "config": {"workload": f"large-{LARGE['mx']}-x{n}", "shots": n, "mx": LARGE["mx"], "mz": LARGE["mz"],
                   "cells_per_shot": inp.cells, "cells_per_level": cells, "tpml": inp.tpml,
                   "levels_per_shot": LARGE["mt2"], "edge": "20-cell PML (the learned edge's fallback)",
                   "l2": "inputs larger than L2 (no flush)", "medium": "shared (one copy on the device)"},
        "shots_per_hour": shots_h(ms_batch, n),
        "single_shot": {"ms_per_level": ms_single, "shots_per_hour": shots_h(ms_single, 1),
                        "gcell_updates_per_s": inp.cells / (ms_single / 1e3) / 1e9},
        "speedup_vs_single_shot_path": shots_h(ms_batch, n) / shots_h(ms_single, 1),
        "roofline": {"bound": "hbm", "kernel": "whole level of every shot", "achieved": gbs, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": gbs / peak, "traffic": None,
                     "alg_bytes_per_level": level_bytes, "march": march},
        "device_memory": {"used_bytes": used, "medium_planes_bytes": plane_bytes,
                          "without_sharing_bytes": used + (n - 1) * plane_bytes},
        "setup_s": {"medium_and_prepare": t_prep, "engines": t_upload},
        "tile_shape": {"units_per_item": shape[0], "waves": shape[1]},
        "core": core,
        "gpu_launches": launches, "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


EDGE = dict(n=512, margin=256, depth_margin=512, levels=2000, f0=20.0, seed=40000)


def _make_edge_pair(item):
    """One (region, wide target) pair of the learned-edge workload (worker)."""
    from fdporo import edge as E
    seed, strip = item
    return E.make_pair(seed, n=EDGE["n"], margin=EDGE["margin"], depth_margin=EDGE["depth_margin"],
                       nsteps=EDGE["levels"], f0=EDGE["f0"], strip=strip)


def run_edge(args) -> None:
    """Learned absorbing edge: networks trained on args.edge_train seeded
    media (region EDGE['n']^2 with a transparent 4-cell strip, target a
    wide run with the reference 20-cell PML), with runs on their own
    between teacher-forced levels; evaluated on args.edge_held other media
    against the strip alone, a 4-cell PML and the reference 20-cell PML.
    Also times a level of the region with the edge against the region
    with the 20-cell PML."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor

    import torch
    from fdporo import edge as E
    from fdporo import job
    L = EDGE["levels"]
    t0 = time.perf_counter()
    train_seeds = [(EDGE["seed"] + k, "plain") for k in range(args.edge_train)]
    held_seeds = [(EDGE["seed"] + 100000 + k, "plain") for k in range(args.edge_held)]
    ctx = mp.get_context("spawn")
    ed = None
    losses = []
    with ProcessPoolExecutor(max_workers=min(8, os.cpu_count() or 1), mp_context=ctx) as pool:
        for epoch in range(args.edge_epochs):
            for k, pair in enumerate(pool.map(_make_edge_pair, train_seeds)):
                if ed is None:
                    ed = E.Edge(scale=E.field_scales(pair, levels=L, every=50), seed=EDGE["seed"])
                    ed.set_output(args.edge_output)
                lr = 1e-3 if args.edge_output == "damp" else 3e-4
                losses += E.train_pair(ed, pair, levels=L, lr=lr, report_every=L, free_every=50, free_run=25)
        train_s = time.perf_counter() - t0
        res = {"strip_alone": [], "learned_edge": [], "pml4": [], "pml20": []}
        for pair in pool.map(_make_edge_pair, held_seeds):
            res["strip_alone"].append(E.evaluate(pair, L))
            res["learned_edge"].append(E.evaluate(pair, L, edge=ed))
            res["pml4"].append(E.evaluate(E.Pair(job.prepare(pair.cfg, pair.medium, "f32"), pair.ext, pair.ox,
                                                 pair.cfg, pair.medium), L))
            res["pml20"].append(E.evaluate(pair, L, tpml=20))
            last = pair
    summary = {k: {m: float(np.mean([r[m] for r in v])) for m in ("reflected_energy", "seismogram_rel_l2")}
               for k, v in res.items()}
    # time per level of the region: learned edge (4-cell strip) vs 20-cell PML
    def level_ms(inp, edge=None):
        eng = job.make_engine(inp)
        if edge is not None:
            edge.attach(eng)
        ext = torch.cuda.ExternalStream(eng.stream())
        eng.time_loop(1, 40)
        eng.prepare_run(320)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        eng.time_loop(41, 40 + 320)
        e1.record(ext)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / 320
        if edge is not None:
            edge.detach(eng)
        eng.close()
        return ms
    ms_edge = level_ms(last.trunc, ed)
    ms_pml = level_ms(E._with_pml(last, 20))
    line = {
        "metric": "learned-edge reflected energy (relative to the target's)", "impl": "gpu",
        "value": summary["learned_edge"]["reflected_energy"], "unit": "ratio", "higher_is_better": False,
        "n_gpus": 1, "dtype": "f32 fields, bf16 networks",
        "data": "synthetic (seeded layered media with Gaussian random fields)",
        "config": {"workload": "learned-edge", "region": EDGE["n"], "target_grid":
                   [EDGE["n"] + 2 * EDGE["margin"], EDGE["n"] + EDGE["depth_margin"]], "levels": L,
                   "train_media": args.edge_train, "held_out_media": args.edge_held, "epochs": args.edge_epochs,
                   "strip_cells": 4, "network": "96-64-64-8 tanh, one per side and depth",
                   "output": args.edge_output},
        "held_out_mean": summary, "train_seconds": train_s, "final_train_loss": losses[-1] if losses else None,
        "level_ms": {"learned_edge_4_cells": ms_edge, "pml_20_cells": ms_pml},
        "region_speedup_vs_pml20": ms_pml / ms_edge,
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--precision", choices=["f32", "f64"], default="f32")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--workload", choices=["layered", "batch", "edge", "large"], default="layered")
    ap.add_argument("--edge-train", type=int, default=32)
    ap.add_argument("--edge-held", type=int, default=8)
    ap.add_argument("--edge-epochs", type=int, default=2)
    ap.add_argument("--edge-output", choices=["damp", "correct"], default="damp")
    ap.add_argument("--shots", type=int, default=BATCH["shots"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-batch", action="store_true", help="leave out the batched-shots leg of the default run")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "edge":
        run_edge(args)
    elif args.workload == "large":
        run_large(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
