#!/usr/bin/env python3
"""Shot-gradients/s of the batched FWI gradient on one GB300.

Workload (default): the batched MCS survey -- 400 x 2000 cells at 12.5 m,
64 shots x 480 channels, 6 s at dt = 1 ms (nt = 6000), 6th-order FD
(acc = 3), 20-cell CPML, snapshots every 10 steps, FP32 stencil and
snapshots, FP64 gradient stack.  One step = one calculate_misfit_gradient
over all 64 shots (forward + L2 misfit + adjoint + imaging + stack).

    python bench.py [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU restatement of the reference solver (the
Fortran reference cannot be compiled here: no Fortran compiler) on all
host cores, one shot per thread, on a bounded number of time steps.
"""
from __future__ import annotations

import argparse
import copy
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "shot-gradients/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["mcs", "single", "was", "mcs-f16", "inversion"], default="mcs",
                    help="mcs: batched MCS survey, 400x2000 cells, 64 shots, 6000 steps (the metric's workload); "
                         "single: one plain shot, 200x400 cells at 25 m, 8th order, 3000 steps; "
                         "was: uneven-window WAS batch; mcs-f16: the MCS survey with snapshots every 4 steps in "
                         "16 bits and checkpointed recomputation under a 120 GB budget; inversion: NLCG inversion "
                         "with frequency continuation (600x3000 cells, 128 shots)")
    ap.add_argument("--errors", action="store_true",
                    help="instead of timing: gradient and misfit errors of the GPU path against an FP64 run of the "
                         "oracle on two shots of the workload at its full grid and record length")
    ap.add_argument("--budget", type=float, default=0.0, help="HBM budget in GB (0: all; mcs-f16: 120)")
    ap.add_argument("--recompute", action="store_true", help="checkpointed recomputation (mcs-f16: on)")
    ap.add_argument("--iters", type=int, default=10, help="inversion: NLCG iterations per band")
    ap.add_argument("--bands", default="3,5,7", help="inversion: low-pass corner frequencies (Hz), one band each")
    ap.add_argument("--order", type=int, default=4, help="inversion: Butterworth order")
    ap.add_argument("--shots", type=int, default=0, help="shots (0 = the workload's: 64 or 30)")
    ap.add_argument("--nt", type=int, default=0, help="time steps (0 = the workload's: 6000 or 12800)")
    ap.add_argument("--snap", choices=["f32", "bf16", "f16"], default=None,
                    help="snapshot form (default f32; mcs-f16: f16)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-path leg")
    ap.add_argument("--profile", type=int, default=0,
                    help="only build the survey and run this many forward time steps (for ncu captures)")
    ap.add_argument("--wave", type=int, default=0, help="shots per wave (0 = tuner)")
    ap.add_argument("--band", type=int, default=0, help="rows per warp work item (0 = tuner)")
    ap.add_argument("--tile-kernel", type=int, default=0, choices=[0, 1, 2],
                    help="two-step tile kernel: 1 register queues, 2 shared-memory queue (0 = tuner)")
    ap.add_argument("--tile-rows", type=int, default=0, help="rows per two-step tile (0 = tuner)")
    ap.add_argument("--tile-edge-rows", type=int, default=0,
                    help="rows of the bottom edge band (0 = tuner; above the model's rows: the last core-height band)")
    a = ap.parse_args()
    if a.workload == "mcs-f16":
        a.snap = a.snap or "f16"
        a.budget = a.budget or 120.0
        a.recompute = True
    a.snap = a.snap or "f32"
    return a


def workload_name(a):
    if a.workload == "single":
        return (f"plain single shot: 200x400 cells @25 m (water over a 1800-4500 m/s gradient with a Gaussian "
                f"anomaly), 1 shot x 200 ch, nt={a.nt} (dt=2 ms), acc=4 (8th order), dPML=20, store_snap=10, "
                f"{a.snap} snapshots, FP64 gradient stack")
    if a.workload == "was":
        return (f"uneven-window WAS batch: 600x6000 cells @25 m crustal model, {a.shots} OBS sources on 30-100 km "
                f"windows, 1200 receivers @125 m, nt={a.nt} (dt=1.5625 ms, the CFL rule; 2.5 ms is unstable), "
                f"acc=3, dPML=20, store_snap=10, {a.snap} snapshots, FP64 gradient stack")
    if a.workload == "mcs-f16":
        return (f"precision form of the batched MCS survey: 400x2000 cells @12.5 m, {a.shots} shots x 480 ch, "
                f"nt={a.nt} (dt=1 ms), acc=3, dPML=20, store_snap=4, {a.snap} snapshots with a power-of-two scale "
                f"per row segment, checkpointed recomputation under a {a.budget:g} GB HBM budget, FP64 stack")
    return (f"batched MCS survey: 400x2000 cells @12.5 m, {a.shots} shots x 480 ch, nt={a.nt} (dt=1 ms), "
            f"acc=3 (6th order), dPML=20, store_snap=10, {a.snap} snapshots, FP64 gradient stack")


def make_workload(a, seed_offset=0):
    from fwi_gb300 import synth
    if a.workload == "single":
        spec, vp_true, vp0 = synth.single_shot()
        a.shots = 1
        a.nt = spec.nt
        return spec, vp_true, vp0
    if a.workload == "inversion":
        a.shots = a.shots or 128
        a.nt = a.nt or 8000
        return synth.inversion_workload(nshots=a.shots, nt=a.nt)
    if a.workload == "was":
        a.shots = a.shots or 30
        spec, vp_true, vp0 = synth.was_batch(seed=3 + seed_offset, nt=a.nt or None, nshots=a.shots)
        a.nt = spec.nt
    else:
        a.shots = a.shots or 64
        a.nt = a.nt or 6000
        spec, vp_true, vp0 = synth.mcs_batch(seed=2 + seed_offset, nshots=a.shots, nt=a.nt,
                                           store_snap=4 if a.workload == "mcs-f16" else 10)
    return spec, vp_true, vp0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile():
    """DRAM bytes per step launch pair from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "step_kernels_mcs64_400x2000.md")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_step_per_shot:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        for line in open(self.f.name):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        loaded = [s for s in sm if s > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
# CPU legs (the oracle is the checker and the CPU baseline, never the product)
# ---------------------------------------------------------------------------

def cpu_sample(spec, vp, nthreads, nt_sample):
    """Time nthreads shot-gradients of the workload, each truncated to
    nt_sample time steps, one shot per thread.  Returns
    (shot-gradients/s scaled to the full nt, seconds, description)."""
    from fwi_gb300.survey import SurveySpec
    from oracle import oracle as O
    shots = []
    for i in range(nthreads):
        s = spec.shots[i % len(spec.shots)]
        src = np.asfortranarray(np.asarray(s.src)[:nt_sample])
        obs = np.asfortranarray(np.random.default_rng(i).standard_normal((nt_sample, len(s.nxRec))).astype(np.float32))
        shots.append(type(s)(x0=s.x0, nx=s.nx, nxSou=s.nxSou, nySou=s.nySou, nxRec=s.nxRec, nyRec=s.nyRec, src=src,
                             obs=obs))
    sub = SurveySpec(ny=spec.ny, nx_model=spec.nx_model, d=spec.d, dt=spec.dt, nt=nt_sample, shots=shots,
                     store_snap=spec.store_snap, acc=spec.acc, dpml=spec.dpml)
    t0 = time.perf_counter()
    O.gradient_batch(sub, vp, step=1, nthreads=nthreads)
    t = time.perf_counter() - t0
    rate = nthreads / (t * (spec.nt / nt_sample))
    if nt_sample >= spec.nt:
        desc = f"{nthreads} full-length shot-gradients of this workload (one per thread)"
    else:
        desc = (f"{nthreads} shot-gradients of this workload (one per thread), each truncated to {nt_sample} of "
                f"{spec.nt} time steps forward and adjoint, scaled by {spec.nt}/{nt_sample}")
    return rate, t, desc


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    # the workload from the oracle's geometry, wavelet and time rules (pinned to
    # the reference's golden vectors): this arm never loads the product library
    from fwi_gb300 import synth
    from oracle import oracle as O
    from oracle import prep as OP
    synth.use_host_functions(O.mcs_geometry, O.ricker, O.time_rules, OP.was_geometry)
    spec, vp_true, vp0 = make_workload(a)
    nthreads = os.cpu_count() or 1
    nt_sample = {"mcs": 100, "mcs-f16": 100, "single": 600}.get(a.workload, 40)
    for _ in range(a.warmup):
        cpu_sample(spec, vp0, nthreads, nt_sample)
    times = []
    rate = None
    desc = ""
    for _ in range(a.steps):
        rate, t, desc = cpu_sample(spec, vp0, nthreads, nt_sample)
        times.append(t)
    per_step = statistics.mean(times)
    value = nthreads / (per_step * (spec.nt / nt_sample))
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload_name(a), "l2": "n/a (CPU)"},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": nthreads, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of solver_acoustic_SS/calculate_misfit_gradient (the Fortran reference "
                    "needs gfortran+MPI, absent here); one shot per host thread, like mpirun -np <cores>"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def run_inversion(a):
    """Config 5: NLCG inversion (FWI.f90's line search, Beta_calculous,
    polyfit) over low-pass bands, all shots batched on the device, with the
    data filtered once per band and resampled to every trial model's dt on the
    device.  Reports the misfit and the model error per iteration and the
    gradient throughput of the whole run."""
    import torch
    import fwi_gb300 as F
    from fwi_gb300 import synth
    from fwi_gb300.inversion import DeviceGradient, RawData, invert

    F.init(0)
    stream = torch.cuda.Stream()
    F.set_stream(stream.cuda_stream)
    snap_form = {"f32": F.SNAP_F32, "bf16": F.SNAP_BF16, "f16": F.SNAP_F16}[a.snap]
    nshots, nt = a.shots or 128, a.nt or 8000
    spec, vp_true, vp0 = synth.inversion_workload(nshots=nshots, nt=nt)
    lam_t, lam0 = synth.lam_from_vp(vp_true), synth.lam_from_vp(vp0)
    # observed data on the true model at the acquisition sampling (untimed)
    sv = F.Survey(spec)
    sv.set_lambda(lam_t)
    sv.run(2)
    obs = np.concatenate([sv.synthetic(i) for i in range(nshots)], axis=1)
    sv.close()
    raw = RawData(obs, F.Ricker_mcs(10.0, spec.dt, nt), spec.dt)
    bands = [(0.0, float(f)) for f in a.bands.split(",")]
    F.set_filter_order(a.order)
    dev = DeviceGradient(spec, raw, snap_form=snap_form)
    clocks = Clocks(0)
    clocks.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lam, log = invert(lam0, dev, bands, a.iters, vp_true=vp_true)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    ck = clocks.stop()
    grads = sum(1 for it in log) + 0.0
    trials = sum(len(it.trials) for it in log)
    calls = dev.calls
    times, axes = dict(dev.times), dev.axes
    dev.close()
    err0 = float(np.linalg.norm(vp0 - vp_true) / np.linalg.norm(vp_true))
    # gradient-equivalents: a step-1 call is one shot-gradient per shot, a
    # line-search trial (forward + misfit) half of one
    geq = nshots * (calls - trials + 0.5 * trials)
    line = {"metric": METRIC, "value": geq / secs, "unit": METRIC, "n_gpus": 1, "steps": len(log), "warmup": 0,
            "ms_per_step": 1e3 * secs / max(len(log), 1), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered model with two low-velocity "
            "lenses; observed data synthesised on the true model)",
            "config": {"workload": f"NLCG inversion: 600x3000 cells @12.5 m, {nshots} MCS shots x 480 ch on "
                       f"their own windows, 8 s records (dt_data=1 ms, nt_data={nt}), low-pass bands "
                       f"{[b[1] for b in bands]} Hz (Butterworth order {a.order}), {a.iters} iterations per "
                       f"band, {a.snap} snapshots, FP64 stack", "bands": bands, "iters_per_band": a.iters},
            "inversion": {"model_error_start": err0, "seconds": secs, "calls": calls, "line_search_trials": trials,
                          "time_axes": axes, "seconds_by_part": times,
                          "iterations": [{"iter": it.iter, "band_hz": it.band[1], "misfit": it.misfit,
                                          "model_error": it.model_error, "step": it.step,
                                          "trials": len(it.trials)} for it in log]},
            "clocks": ck}
    print(json.dumps(line), flush=True)
    return 0


def run_errors(a):
    """Gradient and misfit errors of the GPU path against an FP64 run of the
    oracle (every operation in double precision) on two shots of the workload
    at its full grid and record length, for each snapshot form the workload
    uses.  The observed data are the GPU's FP32 traces on the true model; both
    paths image the starting model.  The GPU gradient is its FP64 stack (before
    the water mask, which both sides would apply alike)."""
    import torch
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp
    from oracle import oracle as O

    F.init(0)
    stream = torch.cuda.Stream()
    F.set_stream(stream.cuda_stream)
    spec, vp_true, vp0 = make_workload(a)
    n = len(spec.shots)
    if a.workload == "was":  # the two narrowest windows (a 100 km window takes the FP64 oracle over 20 minutes)
        order = sorted(range(n), key=lambda i: spec.shots[i].nx)
        pick = sorted(order[:2])
    else:
        pick = sorted({0, n // 2})
    spec.shots = [spec.shots[i] for i in pick]
    lam_t, lam0 = lam_from_vp(vp_true), lam_from_vp(vp0)
    sv = F.Survey(spec)
    sv.set_lambda(lam_t)
    sv.run(2)
    for i, sh in enumerate(spec.shots):
        sh.obs = sv.synthetic(i)
    sv.close()
    forms = {"single": ["f32"], "mcs": ["f32"], "was": ["f32"], "mcs-f16": ["f32", "f16", "bf16"],
             "inversion": ["f32", "f16"]}[a.workload]
    gpu = {}
    for f in forms:
        form = {"f32": F.SNAP_F32, "bf16": F.SNAP_BF16, "f16": F.SNAP_F16}[f]
        sv = F.Survey(spec, snap_form=form)
        sv.set_lambda(lam0)
        m, _ = sv.run(1)
        gpu[f] = (m, sv.stack())
        sv.close()
    vp_ref = np.sqrt(lam0 / np.float32(1000.0)).astype(np.float64)
    t0 = time.perf_counter()
    kern, _, m64, _ = O.gradient_batch(spec, vp_ref, step=1, fp64=True, nthreads=len(spec.shots))
    t_or = time.perf_counter() - t0
    G = np.zeros((spec.ny, spec.nx_model))
    for sh, k in zip(spec.shots, kern):
        G[:, sh.x0:sh.x0 + sh.nx] += sh.grad_weight * k
    mo = float(np.sum(m64))
    # the water mask of the reference's final gradient: rows 1..k of model column j zeroed, k = water_rows[j]
    keep = np.ones_like(G)
    if spec.water_rows is not None:
        keep[np.arange(spec.ny)[:, None] < np.asarray(spec.water_rows)[None, :]] = 0.0

    def rel(g):
        return float(np.linalg.norm(g - G) / np.linalg.norm(G)), \
            float(np.linalg.norm((g - G) * keep) / np.linalg.norm(G * keep))

    out = {}
    for f, (m, g) in gpu.items():
        r_all, r_masked = rel(g)
        out[f] = {"grad_rel_l2": r_all, "grad_rel_l2_water_masked": r_masked, "misfit": m,
                  "misfit_rel": abs(m - mo) / abs(mo)}
    if a.workload == "single":
        # the same solver in FP32 on the CPU (the reference's arithmetic): its own distance from FP64
        k32, _, m32, _ = O.gradient_batch(spec, vp_ref.astype(np.float32), step=1, fp64=False, nthreads=1)
        G32 = np.zeros_like(G)
        for sh, k in zip(spec.shots, k32):
            G32[:, sh.x0:sh.x0 + sh.nx] += sh.grad_weight * k.astype(np.float64)
        r_all, r_masked = rel(G32)
        m32 = float(np.sum(m32))
        out["f32_oracle"] = {"grad_rel_l2": r_all, "grad_rel_l2_water_masked": r_masked, "misfit": m32,
                             "misfit_rel": abs(m32 - mo) / abs(mo)}
    line = {"errors_vs_fp64_oracle": out, "misfit_fp64_oracle": mo, "workload": workload_name(a),
            "shots": [{"index": i, "x0": s.x0, "nx": s.nx} for i, s in zip(pick, spec.shots)], "nt": spec.nt,
            "oracle_seconds": t_or, "oracle_threads": len(spec.shots),
            "how": "GPU: FP32 stencil, the snapshot form named, FP64 stack and misfit; oracle: the same solver "
                   "with every operation in FP64 (CPU); observed data = GPU FP32 traces on the true model"}
    print(json.dumps(line), flush=True)
    return 0


def main():
    a = parse()
    if a.errors:
        return run_errors(a)
    if a.impl == "reference" and a.workload == "inversion":
        print(json.dumps({"impl": "reference", "unavailable": "the inversion workload is an NLCG run; the CPU "
                          "reference arm times the gradient path (the mcs and was workloads)"}))
        return 0
    if a.impl == "reference":
        return run_reference(a)
    if a.workload == "inversion":
        return run_inversion(a)
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl")
    import fwi_gb300 as F
    from fwi_gb300.synth import lam_from_vp

    F.init(local)
    stream = torch.cuda.Stream()
    F.set_stream(stream.cuda_stream)
    snap_form = {"f32": F.SNAP_F32, "bf16": F.SNAP_BF16, "f16": F.SNAP_F16}[a.snap]
    budget = int(a.budget * 1e9)
    # N > 1: one survey of N x (the workload's shots) on one model, shot ranges
    # split over the ranks (each rank holds one copy of the workload's shots),
    # the gradient stack and misfit summed over the ranks in every step
    spec, vp_true, vp0 = make_workload(a)
    global_spec = None
    if world > 1:
        from fwi_gb300 import multi
        global_spec = copy.copy(spec)
        global_spec.shots = list(spec.shots) * world
        spec, _ = multi.shard_spec(global_spec, rank, world)
    lam_true, lam0 = lam_from_vp(vp_true), lam_from_vp(vp0)

    if a.profile:
        sv = F.Survey(spec, snap_form=snap_form, wave_shots=a.wave, band_rows=a.band, hbm_budget=budget,
                      recompute=a.recompute, tile_kernel=a.tile_kernel, tile_rows=a.tile_rows,
                      tile_edge_rows=a.tile_edge_rows)
        sv.set_lambda(lam0)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        sv.time_steps(a.profile)
        p1.record(stream)
        torch.cuda.synchronize()
        ms = p0.elapsed_time(p1) / a.profile
        tb = sv.two_step_bytes()[0]
        print(json.dumps({"profile_steps": a.profile, "ms_per_step": ms, "step_bytes": sv.step_bytes(),
                          "two_step_bytes": tb, "GBps": tb / ms / 1e6, "frac": tb / ms / 1e6 / peaks()[0],
                          "tuning": sv.tuning(), "tiles": [sv.tiles()[0], sv.tiles()[1], sv.edge_tiles()[0]],
                          "tuner_ms_per_pass": {f"{k}/{r}": v for (k, r), v in sv.tiles()[2].items()}}))
        return 0
    # observed data from the true model (untimed setup)
    sv = F.Survey(spec, snap_form=snap_form, wave_shots=a.wave, band_rows=a.band, hbm_budget=budget,
                  recompute=a.recompute, tile_kernel=a.tile_kernel, tile_rows=a.tile_rows,
                      tile_edge_rows=a.tile_edge_rows)
    sv.set_lambda(lam_true)
    sv.run(2)
    for i, sh in enumerate(spec.shots):
        sh.obs = sv.synthetic(i)
    obs_packed = spec.obs_packed()
    sv.set_observed(obs_packed)
    lam0_dev = torch.from_numpy(np.ascontiguousarray(lam0.reshape(-1, order="F"))).cuda()
    sv.set_lambda(lam0_dev.data_ptr())
    grad_dev = torch.zeros(spec.ny * spec.nx_model, dtype=torch.float32, device="cuda")

    grad_host = np.zeros((spec.ny, spec.nx_model), np.float32, order="F")

    def step():
        if world == 1:
            return sv.run_device_grad(1, grad_dev.data_ptr())
        grad_host[...] = 0.0
        return multi.misfit_gradient(sv, global_spec, 1, grad_host)[0]

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(local)
    clocks.start()
    l0 = F.kernel_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(a.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = F.kernel_launch_count() - l0
    t = e0.elapsed_time(e1) / 1e3
    clk = clocks.stop()
    if world > 1:
        tt = torch.tensor([t], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
        torch.distributed.barrier()
    value = world * len(spec.shots) * a.steps / t

    # roofline of the dominant kernel pair (main + bottom step kernels)
    hbm, peak_kind = peaks()
    nsteps = 200
    sv.time_steps(20)
    torch.cuda.synchronize()
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    sv.time_steps(nsteps)
    r1.record(stream)
    torch.cuda.synchronize()
    step_s = r0.elapsed_time(r1) / 1e3 / nsteps
    # the shots of the first wave, which time_steps advances: single-step
    # algorithmic bytes, and those of the two-step passes it runs
    bytes_single = sv.step_bytes()
    bytes_step, tile_bytes_pass = sv.two_step_bytes()
    wave, band = sv.tuning()
    tile_kernel, tile_rows, tile_ms = sv.tiles()
    edge_rows, edge_ms = sv.edge_tiles()
    rc_plan = sv.recompute_plan()
    launch_form, launch_direct_ms, launch_graph_ms = sv.launch_form(1)
    stepping, stepping_ms = sv.stepping()
    achieved = bytes_step / step_s / 1e9
    tr = traffic_from_profile()
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": tr * wave if (tr and a.workload in ("mcs", "mcs-f16")) else None,
            "kernel": ("one time step of all shots of a wave, run as two-step passes: "
                       + ("k_step2s_interior" if tile_kernel == 2 else "k_step2_interior")
                       + f" (model-row interior, two steps per sweep, {tile_rows}-row tiles) beside k_step_strip + "
                       "k_step_bottom + k_step_interior (single-step lists, twice per pass)") if tile_kernel else
                      ("one time step of all shots of a wave, run as single steps (the tuner measured them faster): "
                       + ("k_step_fused (interior, strips and bottom tiles in one launch)" if stepping == "single-fused"
                          else "k_step_interior beside k_step_strip + k_step_bottom")),
            "algorithmic_bytes_per_launch": bytes_step, "avg_launch_ms": step_s * 1e3,
            "single_step_bytes": bytes_single, "single_step_equivalent_GBps": bytes_single / step_s / 1e9,
            "two_step_tile_bytes_per_pass": tile_bytes_pass,
            "peak_kind": f"{peak_kind} copy bandwidth (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
            else "fallback 6.8 TB/s"}
    if a.workload == "single":
        roof["note"] = ("one 200x400 shot: its wavefields (10 x 256 x 512 floats = 5 MB) stay in the 129 MB L2, "
                        "so the step is latency-bound and its fraction of the HBM peak is not meaningful")
    sv.close()
    del sv
    torch.cuda.synchronize()

    # plain GPU path: one shot per survey, one launch per time step, no graph
    plain = None
    if not a.no_plain and rank == 0:
        from fwi_gb300.survey import SurveySpec
        one = SurveySpec(ny=spec.ny, nx_model=spec.nx_model, d=spec.d, dt=spec.dt, nt=spec.nt, shots=[spec.shots[0]],
                         store_snap=spec.store_snap, acc=spec.acc, dpml=spec.dpml, water_rows=spec.water_rows)
        # the 16-bit form compares with the FP32-snapshot plain path
        pv = F.Survey(one, snap_form=F.SNAP_F32 if a.workload == "mcs-f16" else snap_form, graph=False)
        pv.set_lambda(lam0_dev.data_ptr())
        pv.run_device_grad(1, grad_dev.data_ptr())
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        nplain = 2
        for _ in range(nplain):
            pv.run_device_grad(1, grad_dev.data_ptr())
        p1.record(stream)
        torch.cuda.synchronize()
        tp = p0.elapsed_time(p1) / 1e3 / nplain
        plain = {"value": 1.0 / tp, "unit": METRIC, "batched_over_plain": value / world * tp,
                 "how": "same workload one shot at a time, direct kernel launches, no CUDA graph"}
        pv.close()
        del pv
        torch.cuda.synchronize()

    # end to end: the reference-facing batch call with pinned host buffers
    e2e = None
    if not a.no_e2e:
        from fwi_gb300.api import _DescHolder
        pin = lambda n: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
        h_lam = pin(lam0.size)
        h_lam[:] = lam0.reshape(-1, order="F")
        h_grad = pin(spec.ny * spec.nx_model)
        h_obs = pin(obs_packed.size)
        h_obs[:] = obs_packed
        nsrc = sum(np.asarray(s.src).size for s in spec.shots)
        h_src = pin(nsrc)
        h_src[:] = np.concatenate([np.asarray(s.src, np.float32).reshape(-1, order="F") for s in spec.shots])
        dh = _DescHolder(spec, snap_form, F.GRAD_F64, hbm_budget=budget,
                         flags=F.SURVEY_RECOMPUTE if a.recompute else 0, tile_kernel=a.tile_kernel,
                         tile_rows=a.tile_rows, tile_edge_rows=a.tile_edge_rows)
        so = oo = 0
        for i, s in enumerate(spec.shots):
            ns, nr = s.src.size, len(s.nxRec) * spec.nt
            dh.shots[i].src = h_src[so:so + ns].ctypes.data
            dh.shots[i].obs = h_obs[oo:oo + nr].ctypes.data
            so += ns
            oo += nr
        lib = F.load()
        mis = C.c_float(0.0)

        def e2e_step():
            h_grad[:] = 0.0
            rc = lib.fwi_misfit_gradient_batch(C.byref(dh.desc), C.c_void_p(h_lam.ctypes.data), 1, C.byref(mis),
                                               C.c_void_p(h_grad.ctypes.data))
            if rc:
                raise F.FwiError(rc, lib.fwi_last_error().decode())
            if world > 1:  # the ranks' gradients summed (the reference's MPI_REDUCE of Grad)
                tg = torch.from_numpy(h_grad).cuda()
                torch.distributed.all_reduce(tg)
                h_grad[:] = tg.cpu().numpy()
        for _ in range(a.warmup):
            e2e_step()
        torch.cuda.synchronize()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        for _ in range(a.steps):
            e2e_step()
        q1.record(stream)
        torch.cuda.synchronize()
        te = q0.elapsed_time(q1) / 1e3
        if world > 1:
            tt = torch.tensor([te], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            te = float(tt.item())
        bsv = F.batch_survey()
        batch_plan = None
        if bsv is not None:
            bk, br, _ = bsv.tiles()
            batch_plan = {"tile_kernel": bk, "tile_rows": br, "tile_edge_rows": bsv.edge_tiles()[0],
                          "wave_band": list(bsv.tuning()), "time_stepping": bsv.stepping()[0],
                          "launch": list(bsv.launch_form(1))}
        e2e = {"value": world * len(spec.shots) * a.steps / te, "unit": METRIC,
               "h2d_bytes_per_step": int(h_lam.nbytes + h_obs.nbytes + h_src.nbytes + h_grad.nbytes),
               "d2h_bytes_per_step": int(h_grad.nbytes + 8 * sum(len(s.nxRec) for s in spec.shots)),
               "call": "fwi_misfit_gradient_batch (calculate_misfit_gradient drop-in), pinned host buffers",
               "batch_plan": batch_plan}

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        nthreads = os.cpu_count() or 1
        nts = {"mcs": 600, "mcs-f16": 600, "single": spec.nt}.get(a.workload, 150)
        rate, tcpu, desc = cpu_sample(spec, vp0, nthreads, nts)
        cpu = {"value": rate, "unit": METRIC, "cores": nthreads, "kind": "port", "sample": desc,
               "seconds": tcpu}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": t / a.steps * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered model, Ricker sources, "
                "observed data synthesised on the true model)",
                "config": {"workload": workload_name(a), "shots_per_gpu": len(spec.shots), "wave_shots": wave,
                           "band_rows": band, "tile_kernel": tile_kernel, "tile_rows": tile_rows,
                           "tile_edge_rows": edge_rows,
                           "tuner_ms_per_pass": {f"{k}/{r}": v for (k, r), v in tile_ms.items()},
                           "tuner_edge_ms_per_pass": {str(k): v for k, v in edge_ms.items()},
                           "recompute_segment_steps": rc_plan[0], "recompute_segments": rc_plan[1],
                           "launch": {"form": launch_form, "direct_ms": launch_direct_ms,
                                      "graph_replay_ms": launch_graph_ms},
                           "time_stepping": {"form": stepping, "tuner_ms_per_2_steps": stepping_ms},
                           "l2": "inputs larger than L2 (wavefields of all shots of a wave and their snapshots: "
                                 "tens to hundreds of GB)"},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "plain": plain, "gpu_launches": int(launches),
                "clocks": clk}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
