#!/usr/bin/env python3
"""Converged arc-length steps per second on one GB300 (or N replicas).

Default workload: the hinged cylindrical DKT shell panel (R 2540, L 508,
theta 0.2 rad, t 12.7, E 3102.75, nu 0.3) on a 512 x 512 quad mesh: 524,288
triangles, 263,169 joints, 1,575,936 equations (band 3,083), a seeded
four-mode radial imperfection of 0.05 t, centre point load, modified
spherical arc length. One "step" is one converged arc-length increment
(main.c:2647-3134): tangent, LDL^T, predictor and the modified-Newton
corrector iterations to the reference's own convergence test. The headline
leg factors and solves the band in double-word FP32 arithmetic (CB_FP32X2);
the plain FP64 band leg runs beside it on the first increments.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload panel512|panel64|frame|batch]

--workload panel64 measures the 64 x 64 panel (NEQ 24,960) with the FP32
band; --workload frame the nonlinear Newmark workload: the 20 x 20 bay, 30
storey steel frame building (13,671 joints, 38,430 co-rotational 14-DOF
members, warping fixed: NEQ 79,380), seeded band-limited lateral floor
forces, dt 0.005 s; a step is one time step (main.c:3449-3953: full Newton,
the effective stiffness factored every iteration); --workload batch the
batched imperfection sweep.

Under torchrun with N > 1 every rank runs an independent replica of the
analysis on its own GPU (the analysis does not shard); value is the total
steps of all ranks divided by the slowest rank's time.
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
sys.path.insert(0, str(ROOT / "cu-bens_gb300"))

METRIC = "converged load steps/s at 1e-8 residual: learned+mixed vs plain FP64 GPU"
WORKLOAD = "DKT cylindrical panel 64x64 (8192 shells, 4225 joints, NEQ 24960), MSAL"
LARGE_WORKLOAD = ("DKT cylindrical panel 512x512 (524,288 shells, 263,169 joints, NEQ 1,575,936, band 3,083), "
                  "seeded 4-mode imperfection 0.05 t, MSAL")
LARGE_N, LARGE_SEED, LARGE_IMP = 512, 5, 0.05
LARGE_CONTROLS = ("dk -0.05 at the centre joint, alpha 1, psi 0.1, iteopt 6, itemax 100, toldisp 1e-5; force and "
                  "energy criteria off: the reference formulation cannot reach tolforc 1e-8 on the imperfect "
                  "panel (its residual floor is about 2.3e-5 at this dk, approached linearly at 0.4% per "
                  "iteration); every accepted step's |lam q - f| / |lam q| is reported")


def panel_text(n: int = 64):
    from cubens import models
    c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2, toldisp=1e-5,
                            tolforc=1.0, tolener=1.0, itemax=100)
    return models.cylindrical_panel(n, controls=c).text, c


def large_text(n: int = LARGE_N, toldisp: float = 1e-5, n_axial: int | None = None):
    """The 512 x 512 panel (or the same panel on an n x n mesh, or n_axial x n)
    with its controls."""
    from cubens import models
    na = n if n_axial is None else n_axial
    c = models.MsalControls(joint=na // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.05, toldisp=toldisp,
                            tolforc=1.0, tolener=1.0, itemax=100)
    return models.cylindrical_panel(n, seed=LARGE_SEED, imperfection=LARGE_IMP, controls=c, n_axial=n_axial).text


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def bf16_peak():
    """Sustained dense bf16 TFLOP/s (a kernel timed inside a long step)."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if "bf16_tflops_sustained" in d:
            return d["bf16_tflops_sustained"], "measured"
    return 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
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
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg:
        pg.barrier()


def allmax(pg, v: float) -> float:
    if not pg:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def timed_steps(model, k: int):
    """K arc-length steps between two CUDA events on the model's stream."""
    t0 = model.timers()["launches"]
    model.mark(0)
    w0 = time.perf_counter()
    its, res = [], []
    for _ in range(k):
        r = model.step()
        if r.done:
            raise RuntimeError("analysis limits reached inside the timed region")
        its.append(r.iterations)
        res.append(r.residual)
    model.mark(1)
    dev_ms = model.elapsed_ms(0, 1)
    wall_ms = (time.perf_counter() - w0) * 1e3
    launches = model.timers()["launches"] - t0
    return dev_ms, wall_ms, its, res, launches


def cpu_baseline(text: str, target_s: float = 20.0):
    """The oracle port (single thread) on a bounded sample of the same workload:
    the first increment plus as many arc-length steps as fit in ~target_s."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    o = oracle.OracleModel(text)
    t0 = time.perf_counter()
    probe = o.msal_timed(2)  # first increment + one arc step
    per = max(1e-3, probe["t"][1] - probe["t"][0]) if len(probe["t"]) > 1 else 5.0
    steps = int(max(2, min(30, 1 + target_s / per)))
    r = o.msal_timed(steps)
    nstep = len(r["t"]) - 1
    secs = r["t"][-1] - r["t"][0]
    return {"value": nstep / secs, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"oracle port (C restatement, gcc -O2, 1 thread; bit-identical to the reference's own build "
                      f"on the reference's fixtures, which the Arm box cannot build: no reference sources there): "
                      f"first increment untimed, "
                      f"{nstep} arc-length steps timed ({secs:.1f} s), same model",
            "iterations": [int(x) for x in r["its"][1:]], "total_s": time.perf_counter() - t0}


def run_reference(args, world, rank, pg):
    """The reference's CPU implementation of the path (the oracle port: the
    reference compiles on x86 only here) on the host cores, same workload."""
    if rank != 0:
        return
    text, _ = panel_text()
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    o = oracle.OracleModel(text)
    total = 1 + args.warmup + args.steps
    r = o.msal_timed(total)
    if len(r["t"]) < total:
        raise RuntimeError(f"oracle stopped early: {r['error']}")
    t = r["t"]
    secs = t[-1] - t[args.warmup]
    value = args.steps / secs
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "controls": "dk -0.2, toldisp 1e-5"},
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": 1, "kind": "port",
                             "sample": f"first increment + {args.warmup} warm-up steps untimed, "
                                       f"{args.steps} arc-length steps timed"},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FRAME_WORKLOAD = ("frame building 20x20 bays x 30 storeys (13,671 joints, 38,430 frame members, "
                  "NEQ 79,380), nonlinear Newmark dt 0.005")


def frame_text(steps: int, bays=(20, 20, 30)):
    from cubens import models
    return models.frame_building(*bays, steps=steps, dt=0.005, seed=4).text


def frame_cpu_sample(target_s: float = 20.0):
    """The oracle port on a reduced building with the same members, loads and
    controls (10 x 10 bays x 15 storeys, NEQ 10,890, bandwidth 731): whole
    time steps for about target_s, then scaled to the full building by the
    skyline factorisation work n bw^2 of one full-Newton iteration."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    import time as _t
    steps = 3
    o = oracle.OracleModel(frame_text(steps + 1, (10, 10, 15)))
    t0 = _t.perf_counter()
    r = o.newmark(steps)
    secs = _t.perf_counter() - t0
    if r["rc"] < steps:
        raise RuntimeError(f"oracle stopped early: {r['error']}")
    n_s, bw_s = o.neq, 0
    full = oracle.OracleModel(frame_text(2))
    # skyline column heights give the bandwidth of both models
    for mod in (o, full):
        maxa, _ = mod.tangent_fr(*([np.zeros(9 * mod.ne_fr), np.zeros(14 * mod.ne_fr), np.ones(mod.ne_fr),
                                     np.ones(mod.ne_fr)]))
        bw = int(np.max(np.diff(maxa)) - 1)
        if mod is o:
            bw_s = bw
        else:
            bw_f = bw
    scale = (full.neq * bw_f ** 2) / (n_s * bw_s ** 2)
    value = steps / secs / scale
    return {"value": value, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"oracle port (gcc -O2, 1 thread): {steps} time steps of the 10x10x15 building "
                      f"(NEQ {n_s}, bandwidth {bw_s}) in {secs:.1f} s, {np.mean(r['its']):.1f} iterations per step, "
                      f"scaled by n bw^2 to NEQ {full.neq}, bandwidth {bw_f} (x{scale:.1f})"}


def run_frame(args, world, rank, local, pg):
    """Nonlinear Newmark on the frame building. Legs: FGMRES(50) with nodal
    block-Jacobi in FP64 (the plain path), FGMRES with the learned
    preconditioner (trained online on untimed time steps first), and the
    direct band LDL^T (mixed and FP64) for reference. The headline is the
    faster FGMRES leg; every leg solves each Newton step to 1e-12."""
    import cubens
    device = local if world > 1 else 0
    hbm_peak, peak_kind = peaks()
    train = max(args.warmup, 8)
    text = frame_text(train + args.steps + 2)

    def model(kind):
        if kind == "bj":
            return cubens.Model(text, precision=cubens.FP64, device=device, solver=cubens.SOLVER_FGMRES)
        if kind == "mixed":
            return cubens.Model(text, precision=cubens.MIXED, device=device, solver=cubens.SOLVER_FGMRES)
        if kind == "learned":
            m = cubens.Model(text, precision=cubens.FP64, device=device, solver=cubens.SOLVER_FGMRES,
                             precond=cubens.PRECOND_LEARNED)
            m.set_learning(train_steps=train, adam_per_solve=16, lr=1e-3, stall_factor=2.0)
            return m
        return cubens.Model(text, precision=cubens.MIXED if kind == "band_mixed" else cubens.FP64,
                            device=device)

    def timed(m, k, clocks=None):
        barrier(pg)
        l0 = m.timers()["launches"]
        s0 = m.krylov_stats()
        if clocks:
            clocks.start()
        m.mark(0)
        w0 = time.perf_counter()
        its, res = [], []
        for _ in range(k):
            r = m.newmark_step()
            its.append(r.iterations)
            res.append(r.residual)
        m.mark(1)
        dev = m.elapsed_ms(0, 1)
        wall = (time.perf_counter() - w0) * 1e3
        clk = clocks.stop() if clocks else None
        barrier(pg)
        s1 = m.krylov_stats()
        kry = (s1["iterations"] - s0["iterations"]) / max(1, s1["solves"] - s0["solves"])
        return dict(dev_ms=dev, wall_ms=wall, its=its, res=res, clk=clk, launches=m.timers()["launches"] - l0,
                    krylov_steps_per_solve=kry)

    legs = {}
    # FGMRES + block-Jacobi, FP64 (plain)
    m = model("bj")
    m.newmark_begin()
    for _ in range(train):
        m.newmark_step()
    info = m.info
    clocks = ClockSampler(device)
    lb = timed(m, args.steps, clocks)
    ms_spmv, bytes_spmv, flops_spmv = m.profile_kernel(cubens.K_SPMV, reps=20)
    ms_ff, bytes_ff, _ = m.profile_kernel(cubens.K_FRAME_FORCE, reps=5)
    m.close()
    legs["fgmres_block_jacobi_fp64"] = lb
    # FGMRES in mixed precision: FP32 inner FGMRES under an FP64 outer one
    m = model("mixed")
    m.newmark_begin()
    for _ in range(train):
        m.newmark_step()
    lm = timed(m, args.steps, ClockSampler(device))
    lm["stats"] = m.krylov_stats()
    m.close()
    legs["fgmres_mixed"] = lm
    # FGMRES + learned preconditioner (FP32 network in the FP64 FGMRES; block-Jacobi
    # FP64 FGMRES while it trains and whenever it stalls)
    m = model("learned")
    m.newmark_begin()
    for _ in range(train):
        m.newmark_step()
    ll = timed(m, args.steps)
    ll["stats"] = m.krylov_stats()
    ll["ms_train"] = m.timers()["ms_train"]
    m.close()
    legs["fgmres_learned"] = ll
    # direct band LDL^T legs (a few steps: seconds each)
    for kind, k in (("band_mixed", max(1, args.steps // 5)), ("band_fp64", max(1, args.steps // 10))):
        m = model(kind)
        m.newmark_begin()
        m.newmark_step()
        legs[kind] = timed(m, k)
        m.close()
    fg = ("fgmres_block_jacobi_fp64", "fgmres_mixed", "fgmres_learned")
    best = min(fg, key=lambda n: legs[n]["wall_ms"])
    lh = legs[best]
    t_max = allmax(pg, lh["wall_ms"])
    value = world * args.steps / (t_max / 1e3)
    e2e = None
    if not args.skip_e2e:
        barrier(pg)
        w0 = time.perf_counter()
        e = model({"fgmres_block_jacobi_fp64": "bj", "fgmres_mixed": "mixed"}.get(best, "learned"))
        e.newmark_begin()
        d2h = 0
        nst = train + args.steps
        for _ in range(nst):
            e.newmark_step()
            d, _ = e.displacements()
            d2h += d.nbytes
        e2e_s = time.perf_counter() - w0
        h2d = e.info["h2d_bytes"]
        e.close()
        e2e = {"value": world * nst / allmax(pg, e2e_s), "unit": "steps/s", "h2d_bytes_per_step": h2d / nst,
               "d2h_bytes_per_step": d2h / nst,
               "includes": "model_def parse + upload, all time steps from rest (training steps included for "
                           "the learned leg), d read back after every step"}
    if rank != 0:
        return None
    cpu = frame_cpu_sample() if world == 1 and not args.skip_cpu else None
    achieved = bytes_spmv / (ms_spmv * 1e-3) / 1e9

    def summary(leg, k):
        d = {"value": k / (leg["wall_ms"] / 1e3), "ms_per_step": leg["wall_ms"] / k,
             "iterations_per_step": leg["its"], "max_rel_residual": max(leg["res"])}
        if leg.get("krylov_steps_per_solve"):
            d["krylov_steps_per_solve"] = leg["krylov_steps_per_solve"]
        for key in ("stats", "ms_train"):
            if key in leg:
                d[key] = leg[key]
        return d

    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fgmres_block_jacobi_fp64": "f64", "fgmres_mixed": "f32 inner Krylov + f64 outer Krylov/residual"}
        .get(best, "f64 Krylov, f32 network"),
        "data": "synthetic",
        "config": {"workload": FRAME_WORKLOAD, "neq": info["neq"], "nnz": info["nnz"],
                   "node_blocks": info["node_blocks"], "bandwidth": info["bandwidth"], "headline_leg": best,
                   "solver": "FGMRES(50), CGS2, nodal block-Jacobi, relative residual 1e-12 per Newton step; "
                             "mixed: FP32 FGMRES(30) to 1e-4 as the preconditioner of the FP64 FGMRES",
                   "controls": "numopt 0 (beta 0.25, gamma 0.5), lpf 1, toldisp 1e-8, tolener 1e-8",
                   "untimed_steps_before": train, "parallelism": f"replicas x{world}",
                   "l2": "inputs read from HBM each step: CSR matrix and Krylov basis ~0.1 GB, element state "
                         "and band legs > L2",
                   "device_ms_timed": lh["dev_ms"],
                   "mixed_over_fp64": legs["fgmres_block_jacobi_fp64"]["wall_ms"] / legs["fgmres_mixed"]["wall_ms"],
                   "legs": {"fgmres_block_jacobi_fp64": summary(legs["fgmres_block_jacobi_fp64"], args.steps),
                            "fgmres_mixed": summary(legs["fgmres_mixed"], args.steps),
                            "fgmres_learned": summary(legs["fgmres_learned"], args.steps),
                            "band_ldlt_mixed": summary(legs["band_mixed"], max(1, args.steps // 5)),
                            "band_ldlt_fp64": summary(legs["band_fp64"], max(1, args.steps // 10))},
                   "spmv_ms": ms_spmv, "frame_force_ms": ms_ff},
        "roofline": {"kernel": "kry_spmv_kernel (CSR y = A x, FP64 values, 8 lanes per row)", "bound": "hbm",
                     "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "peak_kind": peak_kind,
                     # dram__bytes_read.sum + dram__bytes_write.sum of one launch (ncu capture of the
                     # same command with --steps 4, profiles/fgmres_frame_building.md)
                     "traffic": 39.5e6 + 2.56e3, "traffic_source": "profiles/fgmres_frame_building.md",
                     "bytes_per_launch": bytes_spmv,
                     "ms_per_launch": ms_spmv,
                     "note": "bytes = 12 per stored entry + row pointers + x once + y; timed alone, back to back "
                             "(the matrix is L2-resident between launches)"},
        "cpu_baseline": cpu, "e2e": e2e, "clocks": lh["clk"] or lb["clk"], "gpu_launches": lh["launches"],
    }
    print(json.dumps(line), flush=True)
    return line


def run_reference_frame(args, world, rank, pg):
    if rank != 0:
        return
    cpu = frame_cpu_sample()
    line = {"metric": METRIC, "value": cpu["value"], "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cpu["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": FRAME_WORKLOAD},
            "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


BATCH_WORKLOAD = ("batched imperfection sweep: DKT panels n x n, n drawn from {16,24,...,96} (seeded), "
                  "4-mode imperfection 0.1 t, MSAL dk -0.2, toldisp 1e-4, FP32 tangent/LDL^T + FP64 residual")


def batch_specs(count: int, seed: int = 2024):
    from cubens import models
    out = []
    for i, n in enumerate(models.batch_sizes(count, seed)):
        # the imperfect panels need the displacement tolerance 1e-4: at 1e-5 the
        # reference's own first increment does not converge on most of them
        c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.2, toldisp=1e-4,
                                tolforc=1.0, tolener=1.0, itemax=100)
        out.append(models.cylindrical_panel(n, seed=seed + i, imperfection=0.1, controls=c))
    return out


def _oracle_batch_item(args):
    text, steps = args
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    r = oracle.OracleModel(text).msal_timed(steps)
    return len(r["t"]), (r["t"][-1] - r["t"][0]) if len(r["t"]) > 1 else 0.0, r["t"][0] if len(r["t"]) else 0.0


def batch_cpu_sample(specs, steps: int):
    """The oracle port on the host cores, one process per analysis (the
    reference is single-threaded): a pool of all cores over the first
    instances, each for `steps` arc-length steps; aggregate steps/s."""
    import multiprocessing as mp
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    sample = specs[:cores]
    ctx = mp.get_context("spawn")
    w0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        rs = pool.map(_oracle_batch_item, [(s.text, steps + 1) for s in sample])
    wall = time.perf_counter() - w0
    nsteps = sum(max(0, k - 1) for k, _, _ in rs)
    busy = sum(t for _, t, _ in rs)
    return {"value": nsteps / wall, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"oracle port (gcc -O2), {len(sample)} instances of the sweep in a pool of {cores} "
                      f"processes, {steps} arc-length steps each after the first increment; {nsteps} steps in "
                      f"{wall:.1f} s wall ({busy:.1f} s of step time)"}


def run_batch(args, world, rank, local, pg):
    import cubens
    device = local if world > 1 else 0
    count = args.batch
    specs = batch_specs(count)
    steps = args.steps + 1
    cpu = batch_cpu_sample(specs, min(3, args.steps)) if (rank == 0 and world == 1 and not args.skip_cpu) else None
    c0 = time.perf_counter()
    batch = [cubens.Model(s.text, precision=cubens.MIXED, device=device) for s in specs]
    create_s = time.perf_counter() - c0
    h2d = sum(b.info["h2d_bytes"] for b in batch)
    threads = min(16, os.cpu_count() or 4)
    # warm-up: a separate small batch (first increments of 4 instances)
    warm = [cubens.Model(s.text, precision=cubens.MIXED, device=device) for s in specs[:4]]
    cubens.batch_msal(warm, 1 + args.warmup, threads=threads)
    for w in warm:
        w.close()
    clocks = ClockSampler(device)
    barrier(pg)
    clocks.start()
    w0 = time.perf_counter()
    rc, res = cubens.batch_msal(batch, steps, threads=threads)
    wall = time.perf_counter() - w0
    clk = clocks.stop()
    barrier(pg)
    nconv = sum(len(r["its"]) for r in res)
    t_max = allmax(pg, wall)
    value = world * nconv / t_max
    neqs = [b.info["neq"] for b in batch]
    mem = sum(b.info["device_bytes"] for b in batch)
    launches = sum(b.timers()["launches"] for b in batch)
    for b in batch:
        b.close()
    # the same analyses one after another on one thread
    seq = [cubens.Model(s.text, precision=cubens.MIXED, device=device) for s in specs[:8]]
    w0 = time.perf_counter()
    _, rs = cubens.batch_msal(seq, steps, threads=1)
    seq_wall = time.perf_counter() - w0
    seq_rate = sum(len(r["its"]) for r in rs) / seq_wall
    for b in seq:
        b.close()
    if rank != 0:
        return None
    line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max * 1e3 / max(1, nconv), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 tangent/LDLT + f64 residual",
            "data": "synthetic",
            "config": {"workload": BATCH_WORKLOAD, "instances": count, "steps_per_instance": steps,
                       "neq_min": min(neqs), "neq_max": max(neqs), "host_threads": threads,
                       "device_bytes_total": mem, "status": rc,
                       "sequential_one_thread_steps_per_s": seq_rate,
                       "l2": "working set > L2", "parallelism": f"replicas x{world}"},
            "roofline": None, "cpu_baseline": cpu,
            "e2e": {"value": world * nconv / allmax(pg, create_s + wall), "unit": "steps/s",
                    "h2d_bytes_per_step": h2d / max(1, nconv), "d2h_bytes_per_step": 48,
                    "includes": "model_def parse + upload of every instance, then the batch call (each step's "
                                "record read back)"},
            "clocks": clk, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    return line


def run_reference_batch(args, world, rank, pg):
    if rank != 0:
        return
    cpu = batch_cpu_sample(batch_specs(args.batch), min(3, args.steps))
    line = {"metric": METRIC, "value": cpu["value"], "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cpu["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": BATCH_WORKLOAD, "instances": args.batch},
            "cpu_baseline": cpu, "e2e": {"value": cpu["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                                         "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local, pg):
    import cubens
    text, ctrl = panel_text()
    device = local if world > 1 else 0
    hbm_peak, peak_kind = peaks()

    def analysis(precision):
        m = cubens.Model(text, precision=precision, device=device)
        m.begin()
        for _ in range(args.warmup):
            m.step()
        return m

    # ---- headline: mixed path (FP32 tangent + LDL^T, FP64 residual) ----
    m = analysis(cubens.MIXED)
    clocks = ClockSampler(device)
    barrier(pg)
    clocks.start()
    dev_ms, wall_ms, its, res, launches = timed_steps(m, args.steps)
    clk = clocks.stop()
    barrier(pg)
    t_max = allmax(pg, wall_ms)
    value = world * args.steps / (t_max / 1e3)
    info = m.info

    # per-phase shares (event-timed, separate from the timed region)
    m.reset_timers()
    m.set_timing(True)
    m.step()
    m.set_timing(False)
    tm = m.timers()
    # per-kernel times, each launched alone between CUDA events on the model's
    # stream: the persistent band LDL^T (the dominant kernel of a step), the
    # solve-block formation, the persistent solve (one per Newton iteration)
    # and the shell force kernel
    ms_solve, bytes_solve, _ = m.profile_kernel(cubens.K_SOLVE, reps=50)
    ms_force, bytes_force, flops_force = m.profile_kernel(cubens.K_SHELL_FORCE, reps=20)
    ms_factor, _, flops_factor = m.profile_kernel(cubens.K_FACTOR, reps=3)
    ms_ldlt, bytes_ldlt, flops_ldlt = m.profile_kernel(cubens.K_BAND_LDLT, reps=3)
    ms_blocks, _, flops_blocks = m.profile_kernel(cubens.K_SOLVE_BLOCKS, reps=3)
    m.close()

    # ---- plain FP64 path, same steps ----
    p = analysis(cubens.FP64)
    dev64, wall64, its64, res64, _ = timed_steps(p, args.steps)
    p.reset_timers()
    p.set_timing(True)
    p.step()
    p.set_timing(False)
    tm64 = p.timers()
    p.close()

    # ---- end to end through the public API from host data ----
    e2e = None
    if not args.skip_e2e:
        barrier(pg)
        w0 = time.perf_counter()
        e = cubens.Model(text, precision=cubens.MIXED, device=device)
        e.begin()
        d2h = 0
        for _ in range(args.warmup + args.steps):
            e.step()
            d, lam = e.displacements()
            d2h += d.nbytes + 8
        e2e_s = time.perf_counter() - w0
        h2d = e.info["h2d_bytes"]
        e.close()
        nsteps_e2e = 1 + args.warmup + args.steps
        e2e = {"value": world * nsteps_e2e / allmax(pg, e2e_s), "unit": "steps/s",
               "h2d_bytes_per_step": h2d / nsteps_e2e, "d2h_bytes_per_step": d2h / (nsteps_e2e - 1),
               "includes": "model_def parse + upload, first increment, warm-up and timed steps, "
                           "d read back after every step"}

    line = None
    if rank == 0:
        cpu = cpu_baseline(text) if world == 1 and not args.skip_cpu else None
        achieved = bytes_ldlt / (ms_ldlt * 1e-3) / 1e9
        achieved_solve = bytes_solve / (ms_solve * 1e-3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 tangent/LDLT + f64 residual",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "neq": info["neq"], "bandwidth": info["bandwidth"],
                       "block": info["block"], "nblocks": info["nblocks"],
                       "controls": "dk -0.2, alpha 1, psi 0.1, iteopt 6, itemax 100, toldisp 1e-5 "
                                   "(force/energy criteria off: the reference's DKT drift floor)",
                       "parallelism": f"replicas x{world}", "l2": "working set > L2 (factor blocks "
                       f"{info['device_bytes'] / 1e9:.2f} GB)",
                       "iterations_per_step": its, "max_rel_residual": max(res),
                       "device_ms_timed": dev_ms,
                       "fp64_plain": {"value": args.steps / (wall64 / 1e3), "ms_per_step": wall64 / args.steps,
                                      "iterations_per_step": its64, "max_rel_residual": max(res64)},
                       "mixed_over_fp64": (args.steps / (wall_ms / 1e3)) / (args.steps / (wall64 / 1e3)),
                       "phase_ms_one_step_mixed": {k: round(v, 3) for k, v in tm.items() if k.startswith("ms_")},
                       "phase_ms_one_step_fp64": {k: round(v, 3) for k, v in tm64.items() if k.startswith("ms_")},
                       "solve_ms": ms_solve, "factor_ms": ms_factor,
                       "factor_GFLOPs": flops_factor / (ms_factor * 1e-3) / 1e9,
                       "band_ldlt_ms": ms_ldlt, "band_ldlt_GFLOPs": flops_ldlt / (ms_ldlt * 1e-3) / 1e9,
                       "solve_blocks_ms": ms_blocks,
                       "solve_blocks_GFLOPs": flops_blocks / (ms_blocks * 1e-3) / 1e9,
                       "shell_force_ms": ms_force,
                       "shell_force_GBps": bytes_force / (ms_force * 1e-3) / 1e9,
                       "shell_force_fp64_GFLOPs": flops_force / (ms_force * 1e-3) / 1e9},
            "roofline": {"kernel": (f"factor_cluster_kernel (band LDL^T, FP32, one {info['factor_cluster']}-CTA "
                                    "thread-block cluster, the band's window in distributed shared memory, one "
                                    "cluster barrier per 32-column panel)") if info.get("factor_cluster") else
                                   "factor_f32_kernel (persistent band LDL^T, FP32, one grid barrier per 32-column "
                                   "panel)",
                         "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                         # dram__bytes_read.sum + dram__bytes_write.sum of one launch of the grid factor
                         # (ncu capture, profiles/factor_f32_kernel_panel64.md); the cluster factor has none
                         "traffic": None if info.get("factor_cluster") else 39.74e6 + 3.65e6,
                         "traffic_source": "profiles/factor_f32_kernel_panel64.md",
                         "bytes_per_launch": bytes_ldlt, "ms_per_launch": ms_ldlt,
                         "note": "latency-bound: 780 dependent panels; bytes = the band read and written "
                                 "once; FP32 FMA work n*bw^2/2 per launch"},
            "roofline_solve": {"kernel": "solve_kernel<float> (persistent block-bidiagonal solve, FP32)",
                               "bound": "hbm", "achieved": achieved_solve, "peak": hbm_peak, "unit": "GB/s",
                               "frac": achieved_solve / hbm_peak, "peak_kind": peak_kind,
                               # one launch's dram__bytes_read.sum + dram__bytes_write.sum (ncu capture of
                               # the same command with --steps 3, profiles/factor_f32_kernel_panel64.md)
                               "traffic": 247.31e6 + 4.44e6, "traffic_source": "profiles/factor_f32_kernel_panel64.md",
                               "bytes_per_launch": bytes_solve, "ms_per_launch": ms_solve},
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")} if cpu else None,
            "e2e": e2e,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(line), flush=True)
    return line


def large_cpu_sample(n_sample: int = 128, steps: int = 2):
    """The oracle port (single thread, the reference is serial) on the same
    panel at n_sample x n_sample: the first increment untimed, then `steps`
    arc-length steps timed; scaled to the 512 x 512 panel by the skyline
    factorisation work n bw^2 (the factorisation dominates a step once the
    band is wide: three or four iterations per step here). A step of the
    full panel takes about an hour and a half on one core, so it is
    extrapolated."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    oracle.build()
    o = oracle.OracleModel(large_text(n_sample))
    t0 = time.perf_counter()
    r = o.msal_timed(1 + steps)
    if len(r["t"]) < 1 + steps:
        raise RuntimeError(f"oracle stopped early: {r['error']}")
    secs = r["t"][-1] - r["t"][0]
    wall = time.perf_counter() - t0

    def neq_bw(n):
        # hinged straight edges: 3 translations of 2 (n + 1) joints fixed; row-major joint numbering
        return 6 * (n + 1) ** 2 - 6 * (n + 1), 6 * (n + 2) - 1

    ns, bs = neq_bw(n_sample)
    nf, bf = neq_bw(LARGE_N)
    scale = (nf * bf ** 2) / (ns * bs ** 2)
    per_step = secs / steps * scale
    return {"value": 1.0 / per_step, "unit": "steps/s", "cores": 1, "kind": "port",
            "sample": f"oracle port (C restatement of the reference, gcc -O2, 1 thread; bit-identical to the "
                      f"reference's own build on its fixtures; the Arm box has no reference sources): the same "
                      f"panel on a "
                      f"{n_sample}x{n_sample} mesh (NEQ {ns}), first increment untimed, {steps} arc-length steps "
                      f"in {secs:.1f} s ({[int(x) for x in r['its'][1:]]} iterations), scaled by n bw^2 to NEQ "
                      f"{nf} (x{scale:.0f}): extrapolated, {per_step / 3600:.2f} h per step",
            "total_s": wall}


def run_large(args, world, rank, local, pg):
    """The 512 x 512 panel: the double-word FP32 band (headline), the plain
    FP64 band on the first increments, end to end through the public API."""
    import cubens
    device = local if world > 1 else 0
    hbm_peak, peak_kind = peaks()
    text = large_text()
    total = 1 + args.warmup + args.steps
    # ---- headline: created from the model_def text (the end-to-end clock starts), first
    #      increment, warm-up, the timed steps; d read back after every increment ----
    barrier(pg)
    w_e2e = time.perf_counter()
    m = cubens.Model(text, precision=cubens.FP32X2, device=device, band_solve=1)
    info = m.info
    recs = []

    def record(r):
        d, lam = m.displacements()
        recs.append({"lam": r.lam, "its": r.iterations, "res": r.residual, "dk": r.dk, "d": d})

    record(m.begin())
    for _ in range(args.warmup):
        record(m.step())
    clocks = ClockSampler(device)
    barrier(pg)
    clocks.start()
    l0 = m.timers()["launches"]
    m.mark(0)
    w0 = time.perf_counter()
    for _ in range(args.steps):
        r = m.step()
        if r.done:
            raise RuntimeError("analysis limits reached inside the timed region")
        record(r)
    m.mark(1)
    dev_ms = m.elapsed_ms(0, 1)
    wall_ms = (time.perf_counter() - w0) * 1e3
    launches = m.timers()["launches"] - l0
    e2e_s = time.perf_counter() - w_e2e
    clk = clocks.stop()
    barrier(pg)
    t_max = allmax(pg, wall_ms)
    value = world * args.steps / (t_max / 1e3)
    d2h = sum(x["d"].nbytes + 8 for x in recs)
    e2e = {"value": world * total / allmax(pg, e2e_s), "unit": "steps/s",
           "h2d_bytes_per_step": info["h2d_bytes"] / total, "d2h_bytes_per_step": d2h / total,
           "includes": "model_def parse + upload, first increment, warm-up and timed increments, d read back "
                       "after every increment (host buffers, C ABI through ctypes)"}
    # per-phase times of one more increment, then the dominant kernels alone
    m.reset_timers()
    m.set_timing(True)
    m.step()
    m.set_timing(False)
    tm = m.timers()
    ms_solve, bytes_solve, _ = m.profile_kernel(cubens.K_SOLVE, reps=5)
    ms_force, bytes_force, flops_force = m.profile_kernel(cubens.K_SHELL_FORCE, reps=20)
    ms_ldlt, bytes_ldlt, flops_ldlt = m.profile_kernel(cubens.K_BAND_LDLT, reps=1)
    m.close()
    # ---- plain FP64 band on the first increments (a step is about half a minute) ----
    k64 = max(1, min(args.steps, args.fp64_steps))
    p = cubens.Model(text, precision=cubens.FP64, device=device, band_solve=1)
    p64 = [p.begin()]
    d64 = [p.displacements()[0]]
    w0 = time.perf_counter()
    for _ in range(k64):
        p64.append(p.step())
        d64.append(p.displacements()[0])
    wall64 = (time.perf_counter() - w0) * 1e3
    p.reset_timers()
    p.set_timing(True)
    p.step()
    p.set_timing(False)
    tm64 = p.timers()
    p.close()
    krylov = krylov_legs(device, args.krylov_maxit) if args.krylov_maxit > 0 else None
    if rank != 0:
        return None
    # per-increment error of the headline leg against the FP64 leg (same increments)
    err = []
    for k, (rr, dd) in enumerate(zip(p64, d64)):
        x = recs[k]
        err.append({"increment": k, "iterations_fp32x2": x["its"], "iterations_fp64": rr.iterations,
                    "lam_rel_err": abs(x["lam"] - rr.lam) / abs(rr.lam),
                    "d_rel_err": float(np.linalg.norm(x["d"] - dd) / np.linalg.norm(dd))})
    cpu = large_cpu_sample() if world == 1 and not args.skip_cpu else None
    timed = recs[1 + args.warmup:]
    n, bw = info["neq"], info["bandwidth"]
    fma = n * bw * bw / 2.0                        # band LDL^T multiply-adds per factorisation
    tc_flops = fma * 21 * 2.0                      # bfloat16 slice products executed on the tensor cores
    tc_peak, tc_peak_kind = bf16_peak()
    achieved = bytes_ldlt / (ms_ldlt * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 forces/residual/arc-length; f64 tangent; band LDL^T in double-word f32 (~48-bit) with its "
                 "trailing update as bf16 slice products on the tensor cores (exact f32 accumulation); solves in "
                 "double-word f32",
        "data": "synthetic",
        "config": {"workload": LARGE_WORKLOAD, "neq": n, "bandwidth": bw, "seed": LARGE_SEED,
                   "imperfection": f"{LARGE_IMP} t, modes (1,1),(1,2),(2,1),(2,2)", "controls": LARGE_CONTROLS,
                   "parallelism": f"replicas x{world}",
                   "l2": f"working set > L2: {info['device_bytes'] / 1e9:.1f} GB on the device (the band "
                         f"{8 * n * (bw + 5) / 1e9:.1f} GB), streamed by every factorisation and solve",
                   "iterations_per_step": [x["its"] for x in timed],
                   "max_rel_residual": max(x["res"] for x in timed),
                   "residual_per_step": [x["res"] for x in timed],
                   "lam_per_step": [x["lam"] for x in timed],
                   "device_ms_timed": dev_ms,
                   "error_vs_fp64_gpu": err,
                   "fp64_plain": {"value": k64 / (wall64 / 1e3), "ms_per_step": wall64 / k64, "steps": k64,
                                  "iterations_per_step": [x.iterations for x in p64[1:]],
                                  "max_rel_residual": max(x.residual for x in p64[1:]),
                                  "phase_ms_one_step": {k: round(v, 1) for k, v in tm64.items()
                                                        if k.startswith("ms_")}},
                   "fp32x2_over_fp64": (args.steps / (wall_ms / 1e3)) / (k64 / (wall64 / 1e3)),
                   "fgmres_legs": krylov,
                   "phase_ms_one_step": {k: round(v, 1) for k, v in tm.items() if k.startswith("ms_")},
                   "band_ldlt_ms": ms_ldlt, "band_ldlt_fma_per_s": fma / (ms_ldlt * 1e-3),
                   "solve_ms": ms_solve, "shell_force_ms": ms_force,
                   "shell_force_GBps": bytes_force / (ms_force * 1e-3) / 1e9,
                   "fp32_band_ldlt": "diverges at this size (first increment: lambda 615 after the first solve "
                                     "against 81.45, no convergence in 100 iterations); not a leg"},
        "roofline": {"kernel": "factor_dw_tc_kernel (persistent band LDL^T in double-word FP32, trailing update "
                               "on the tensor cores: 21 bfloat16 slice products per multiply-add, mma.sync)",
                     "bound": "tensor", "achieved": tc_flops / (ms_ldlt * 1e-3) / 1e12, "peak": tc_peak,
                     "unit": "TFLOP/s", "frac": tc_flops / (ms_ldlt * 1e-3) / 1e12 / tc_peak,
                     "peak_kind": f"{tc_peak_kind} (cuBLAS bf16, sustained: the kernel runs inside a long step)",
                     "traffic": (TRAFFIC_TC_512x32 * (n * (bw + 5)) / (101376 * 3088)) if TRAFFIC_TC_512x32 else None,
                     "traffic_source": "profiles/factor_dw_tc_kernel_panel512.md (one launch on the 512 x 32 "
                                       "panel, the same band, scaled by n ld)",
                     "work": f"n bw^2 / 2 = {fma:.3e} double-word multiply-adds x 21 slice products x 2 flops",
                     "ms_per_launch": ms_ldlt,
                     "mma_sync_ceiling_tflops": MMA_SYNC_TFLOPS,
                     "frac_of_mma_sync_ceiling": tc_flops / (ms_ldlt * 1e-3) / 1e12 / MMA_SYNC_TFLOPS,
                     "note": "mma.sync (bf16, m16n8k16) peaks near 600 TFLOP/s on GB300, below the tcgen05 rate "
                             "that cuBLAS reaches; the band's bytes (read and written once) are in roofline_hbm"},
        "roofline_hbm": {"kernel": "factor_dw_tc_kernel", "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                         "bytes_per_launch": bytes_ldlt},
        "fp64_equivalent": {"kernel": "factor_dw_tc_kernel", "achieved": 2 * fma / (ms_ldlt * 1e-3) / 1e12,
                            "unit": "TFLOP/s of ~48-bit multiply-adds (2 per)",
                            "fp64_band_factor_tflops": 2 * fma / (tm64["ms_factor"] * 1e-3) / 1e12,
                            "note": "the same factorisation in native FP64 on GB300's FP64 pipe (the plain leg)"},
        "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")} if cpu else None,
        "e2e": e2e, "clocks": clk, "gpu_launches": launches,
    }
    print(json.dumps(line), flush=True)
    return line


def krylov_legs(device: int, maxit: int):
    """The FGMRES(50) legs on the 512 x 512 panel's first increment, with a
    bounded Arnoldi budget per solve: nodal block-Jacobi in FP64, and the
    learned preconditioner with the mixed-precision inner solver. Neither
    can converge there (the DKT panel's bending makes the block-Jacobi-scaled
    tangent's condition number grow as n^4), so each leg reports how far its
    solves get instead of a step rate, and the learned+mixed over plain FP64
    ratio stays undefined."""
    import cubens
    from cubens import models
    n = LARGE_N
    c = models.MsalControls(joint=n // 2 * (n + 1) + n // 2 + 1, direction=3, dk=-0.05, toldisp=1e-5,
                            tolforc=1.0, tolener=1.0, itemax=2, submax=0)
    text = models.cylindrical_panel(n, seed=LARGE_SEED, imperfection=LARGE_IMP, controls=c).text
    out = {"restart": 50,
           "controls": "the config's first increment with itemax 2 (two corrector iterations) and no subdivision"}
    # the mixed leg's outer steps each run an FP32 FGMRES(30) inner solve of up to 400 steps
    for name, lim, kw in (("fp64_block_jacobi", maxit, dict(precision=cubens.FP64)),
                          ("mixed_learned", max(1, maxit // 20),
                           dict(precision=cubens.MIXED, precond=cubens.PRECOND_LEARNED))):
        w0 = time.perf_counter()
        m = cubens.Model(text, solver=cubens.SOLVER_FGMRES, maxit=lim, device=device, **kw)
        w1 = time.perf_counter()
        try:
            r = m.begin()
            status = f"first increment converged in {r.iterations} iterations"
        except cubens.CubensError as e:
            status = f"first increment not converged ({e})"
        w2 = time.perf_counter()
        s = m.krylov_stats()
        m.close()
        out[name] = {"status": status, "arnoldi_limit_per_solve": lim, "create_s": round(w1 - w0, 2),
                     "first_increment_s": round(w2 - w1, 2),
                     "solves": s["solves"], "arnoldi_steps": s["iterations"],
                     "inner_fp32_steps": s["inner_iterations"], "unconverged_solves": s["unconverged"],
                     "last_solve_rel_residual": s["last_residual"],
                     "train_steps": s["train_steps"], "train_loss": s["train_loss"],
                     "learned_solves": s["learned_solves"]}
    out["learned_mixed_over_plain_fp64"] = None
    return out


def run_reference_large(args, world, rank, pg):
    """The reference's CPU path (the oracle port) on the host, extrapolated
    from the same panel on a 128 x 128 mesh (a step of the 512 x 512 panel is
    about an hour and a half on one core)."""
    if rank != 0:
        return
    cpu = large_cpu_sample()
    line = {"metric": METRIC, "value": cpu["value"], "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / cpu["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": LARGE_WORKLOAD, "controls": LARGE_CONTROLS},
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cpu["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# dram__bytes_read.sum + dram__bytes_write.sum of one factor_dw_tc_kernel launch on the 512 x 32
# panel (NEQ 101,376, ld 3,088), from profiles/factor_dw_tc_kernel_panel512.md
TRAFFIC_TC_512x32 = 2503401728 + 6141808128
# bf16 mma.sync m16n8k16 throughput measured on GB300 (all SMs, independent accumulators)
MMA_SYNC_TFLOPS = 600.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the CPU-baseline sample (profiling runs)")
    ap.add_argument("--skip-e2e", action="store_true", help="omit the end-to-end leg (profiling runs)")
    ap.add_argument("--workload", choices=["panel512", "panel64", "frame", "batch"], default="panel512",
                    help="panel512: MSAL DKT panel 512x512, 1.58M equations (default); panel64: the 64x64 "
                         "panel; frame: nonlinear Newmark frame building; batch: the batched imperfection sweep")
    ap.add_argument("--factor-only", default="", metavar="N[xA]",
                    help="profiling: the FP32x2 band LDL^T of the same panel on an N x N mesh, or A axial by N "
                         "circumferential divisions (the band of the N x N panel with fewer equations): first "
                         "increment, then one factorisation alone; no JSON line")
    ap.add_argument("--force-only", type=int, default=0, metavar="N",
                    help="profiling: shell_forces_kernel on the same panel on an N x N mesh (first increment, "
                         "then 20 launches alone); no JSON line")
    ap.add_argument("--factor-kernel", type=int, default=0,
                    help="--factor-only: 0 the tensor-core double-word factor, 1 the FP32-pipe one")
    ap.add_argument("--fp64-steps", type=int, default=2,
                    help="panel512: timed increments of the plain FP64 leg (about half a minute each)")
    ap.add_argument("--batch", type=int, default=48, help="instances of the batch workload")
    ap.add_argument("--krylov-maxit", type=int, default=1000,
                    help="Arnoldi steps per solve of the panel512 FGMRES legs (0: omit them)")
    args = ap.parse_args()
    if args.factor_only:
        import cubens
        nf, _, na = args.factor_only.partition("x")
        m = cubens.Model(large_text(int(nf), n_axial=int(na) if na else None), precision=cubens.FP32X2,
                         band_solve=1, factor_kernel=args.factor_kernel)
        m.begin()
        ms, _, fl = m.profile_kernel(cubens.K_BAND_LDLT, reps=1)
        print(f"band LDL^T, NEQ {m.neq}, band {m.info['bandwidth']}: {ms:.1f} ms, "
              f"{fl / 2 / (ms * 1e-3) / 1e12:.3f} T double-word multiply-adds/s", flush=True)
        return
    if args.force_only:
        import cubens
        m = cubens.Model(large_text(args.force_only), precision=cubens.FP32X2, band_solve=1)
        m.begin()
        ms, nbytes, fl = m.profile_kernel(cubens.K_SHELL_FORCE, reps=20)
        print(f"shell_forces_kernel, {m.info['ne_sh']} elements: {ms * 1e3:.1f} us, "
              f"{nbytes / (ms * 1e-3) / 1e9:.0f} GB/s of {nbytes / m.info['ne_sh']:.0f} B per element, "
              f"{fl / (ms * 1e-3) / 1e12:.3f} TFLOP/s FP64 (estimated flops)", flush=True)
        return
    world, rank, local, pg = dist_setup(args.gpus)
    if args.workload == "batch":
        if args.impl == "reference":
            run_reference_batch(args, world, rank, pg)
        else:
            run_batch(args, world, rank, local, pg)
    elif args.workload == "frame":
        if args.impl == "reference":
            run_reference_frame(args, world, rank, pg)
        else:
            run_frame(args, world, rank, local, pg)
    elif args.workload == "panel64":
        if args.impl == "reference":
            run_reference(args, world, rank, pg)
        else:
            run_ours(args, world, rank, local, pg)
    elif args.impl == "reference":
        run_reference_large(args, world, rank, pg)
    else:
        run_large(args, world, rank, local, pg)
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
