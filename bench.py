#!/usr/bin/env python3
"""Benchmark of the per-snapshot reionization grid step on GB300.

Workload (evolve_512): 512^3 cells, L = 200 Mpc/h, seed 2, fields grown
linearly with the growth factor over 20 snapshots z = 15 -> 6; every snapshot
runs the full step ComputeTs (40 shells) -> find_HII_bubbles (recombinations,
41 radii, 5 fields) -> 21 cm brightness temperature.  A benchmark "step" is one
snapshot.  Inputs are seeded synthetic grids (no simulation data).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  `value` is ms per snapshot with the inputs resident in
HBM (device entry points); `e2e` is the same metric through the host-pointer
entry point mx_step with pinned host buffers (copies inside the timed
region); `roofline` reports the dominant kernel's achieved HBM bandwidth from
CUDA events; `cpu_baseline` is the CPU oracle on the host cores.  With N > 1
(torchrun) the ranks run independent replicas (no data exchange).
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "ms/snapshot at 512^3 (ComputeTs + find_HII_bubbles + 21cm box)"
UNIT = "ms/snapshot"
REION_EFF = 1.0 / 0.15714 * 4000.0 / (1.0 - 0.75 * 0.24)
FESC = 0.01
# DRAM bytes (read + write) per algorithmic byte of each kernel, from one
# `ncu --set full` capture of each kernel at 256^3 (profiles/*_256.md: `python
# bench.py --grid 256 --steps 2 --warmup 1 --no-cpu --no-e2e --no-adjoint
# --no-batch --no-plain --no-graph` with MX_MAX_BATCH_SPECTRA=20, one to two
# launches per kernel).  A kernel's DRAM traffic grows with the spectra (or
# cells) it processes, so the traffic of a 512^3 launch is the ratio times the
# launch's algorithmic bytes.  The transforms also move the row padding of
# the spectra (rows of 144 complex values for 129 at 256^3, 272 for 257 at
# 512^3): PAD_512_OVER_256 rescales that share of their ratios.  The
# threshold z-pass also reads the state (xH, z_at_ionization: 8 bytes per
# cell) at the start of every launch; the algorithmic model counts it once per
# call, so it is added per launch (THRESHOLD_STATE_BYTES_PER_CELL).
_C256, _N256 = 256 * 256 * 129, 256 ** 3
PAD_512_OVER_256 = (272 / 257) / (144 / 129)
DRAM_PER_ALGORITHMIC = {
    # 5 unfiltered spectra read, 20 written; algorithmic 8 C G (1 + n_radii)
    "fft_x_filter": (0.377542e9 + 1.452510e9) / (8 * _C256 * 5 * 5) * PAD_512_OVER_256,
    # 20 spectra read and written; algorithmic 16 C per spectrum
    "fft_y": (1.509980e9 + 1.447947e9) / (16 * _C256 * 20) * PAD_512_OVER_256,
    # 20 spectra read (the state read of 8 B per cell taken out)
    "fft_z_threshold": (1.644234e9 + 3.307264e6 - 8 * _N256) / (8 * _C256 * 20) * PAD_512_OVER_256,
    # 19 shells: spectra read, shells written
    "fft_z_store": (1.434571e9 + 1.234466e9) / ((8 * _C256 + 4 * _N256) * 19),
    "k_evolve": (2.887466e9 + 0.196168e9) / (46 * 4 * _N256),
}
THRESHOLD_STATE_BYTES_PER_CELL = 8


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-adjoint", action="store_true",
                    help="also time the 48-box batch with the adjoint of every box (Python workers)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="time the device step uncaptured")
    ap.add_argument("--adjoint-grid", type=int, default=256)
    return ap.parse_args(argv)


def workload_for(grid: int):
    from meraxes_gb300.params import workload

    w = workload("evolve_512", grid if grid != 512 else None)
    w.params.reion_efficiency = REION_EFF
    w.fesc = FESC
    return w


# ----------------------------------------------------------------- distributed
def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world: int, backend: str):
    import torch.distributed as dist

    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms_local: float, steps: int, world: int, device=None) -> float:
    """Whole-job ms per snapshot over N independent replicas: every rank ran
    `steps` snapshots; the job's time is the slowest rank's."""
    return max_over_ranks(ms_local, world, device) / (steps * world)


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
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
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------- synthetic
def make_device_fields(w, snapshots, device):
    """Seeded inputs of the given snapshots, generated on the GPU with the
    recipe of meraxes_gb300.synthetic (PCG64 white noise, P(k) filtering,
    growth-factor scaling, stellar mass and SFR grids) in the PADDED layout."""
    import torch

    from meraxes_gb300.params import growth_factor, sfr_timescale_internal_myr

    p = w.params
    D, L = p.grid_dim, p.box_size
    H = D // 2 + 1
    rng = np.random.default_rng(w.seed)
    noise = torch.from_numpy(rng.standard_normal((D, D, D))).to(device)
    fk = torch.fft.rfftn(noise)
    del noise
    kf = 2.0 * np.pi / L
    kx = torch.fft.fftfreq(D, d=1.0 / D, device=device, dtype=torch.float64) * kf
    kz = torch.fft.rfftfreq(D, d=1.0 / D, device=device, dtype=torch.float64) * kf
    k2 = kx[:, None, None] ** 2 + kx[None, :, None] ** 2 + kz[None, None, :] ** 2
    kny = np.pi * D / L
    pk = torch.where(k2 > 0, torch.exp(-k2 / kny ** 2) / torch.where(k2 > 0, k2, torch.ones_like(k2)),
                     torch.zeros_like(k2))
    fk *= torch.sqrt(pk)
    del pk, k2
    base = torch.fft.irfftn(fk, s=(D, D, D))
    del fk
    base *= 0.6 / base.std()
    d_norm = growth_factor(w.redshifts[w.snapshots[-1]], p)
    t20 = sfr_timescale_internal_myr(20.0, p)
    out = {}
    for s in snapshots:
        d = torch.clamp(base * (growth_factor(w.redshifts[s], p) / d_norm), min=-0.99).float()
        dd = d.double()
        stars = torch.where(dd > 0.5, 1e-3 * torch.exp(2.0 * dd), torch.zeros_like(dd))
        sfr = (stars / t20).float()
        grids = {}
        for name, val in (("deltax", d), ("stars", (w.fesc * stars.float().double()).float()),
                          ("weighted_sfr", (w.fesc * sfr.double()).float()), ("sfr", sfr)):
            t = torch.zeros((D, D, 2 * H), dtype=torch.float32, device=device)
            t[:, :, :D] = val
            grids[name] = t
        out[s] = grids
        del d, dd, stars
    del base
    return out


def history_buffer(fields, snapshots, n_hist, D, device):
    """All SFR grids in reverse snapshot order, so that the contiguous slices
    [s-0, s-1, ...] for any snapshot are a view (padded with zero slices)."""
    import torch

    H = D // 2 + 1
    P = D * D * 2 * H
    smax = max(snapshots)
    buf = torch.zeros((smax + 1 + n_hist, P), dtype=torch.float32, device=device)
    for s in snapshots:
        buf[smax - s] = fields[s]["sfr"].reshape(-1)
    return buf, smax


def state_grids(p, z_prev, device):
    import torch

    from meraxes_gb300 import synthetic as syn

    st = syn.initial_state(p, z_prev)
    return {k: torch.from_numpy(v).to(device) for k, v in st.items()}


# -------------------------------------------------------------------- arms
def time_evolution(step, w, fields, hist, smax, warm, timed, device, world, local, profile=False):
    """Runs the warm-up snapshots, resets the state, then times the
    snapshots `timed` of one evolution from the initial state (CUDA events
    on the default stream, barrier + synchronize on both sides).  Where the
    timed list wraps past the last snapshot, the state is reset to the
    initial state (a device copy inside the timed region) so that every
    snapshot runs on the state of its own evolution."""
    import torch

    n_hist = step.n_sfr_histories
    state0 = state_grids(w.params, w.redshifts[0], device)
    state = {k: v.clone() for k, v in state0.items()}

    def grids_for(s):
        g = dict(state)
        g.update(fields[s])
        g["sfr_histories"] = hist[smax - s: smax - s + n_hist]
        return g

    def reset():
        for k, v in state0.items():
            state[k].copy_(v)

    for s in warm:
        if s == 0:
            reset()
        step.step(s, grids_for(s))
    reset()
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(local)
    clocks.start()
    if profile:
        step.profile(True)
    launches = 0
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier(world)
    t0.record()
    glob = None
    for i, s in enumerate(timed):
        if s == 0 and i > 0:
            reset()
        glob = step.step(s, grids_for(s))
        launches += step.last_launches
    t1.record()
    torch.cuda.synchronize()
    barrier(world)
    ms = t0.elapsed_time(t1)
    clk = clocks.stop()
    kstats = None
    if profile:
        kstats = step.profile_read()
        step.profile(False)
    return ms, launches, glob, clk, kstats


def run_plain_gpu(args, w, fields, hist, smax, warm, timed, device, world, local):
    """The "plain GPU" comparator: the same evolution through the same entry
    points with the transforms of a plain GPU port (MX_TRANSFORM=cufft: one
    cuFFT R2C per field, then per radius and field a filter kernel, a cuFFT
    C2R and separate clamp/threshold kernels, the loop structure of the
    reference)."""
    from meraxes_gb300.api import ReionGridStep

    old = os.environ.get("MX_TRANSFORM")
    os.environ["MX_TRANSFORM"] = "cufft"
    try:
        step = ReionGridStep(w.params, w.redshifts)
    finally:
        if old is None:
            os.environ.pop("MX_TRANSFORM", None)
        else:
            os.environ["MX_TRANSFORM"] = old
    ms, launches, glob, clk, _ = time_evolution(step, w, fields, hist, smax, warm, timed, device, world, local)
    step.close()
    return {"value": round(replica_value(ms, len(timed), world, device), 3), "unit": UNIT,
            "transform": "cuFFT R2C/C2R + per-radius filter and threshold kernels (MX_TRANSFORM=cufft)",
            "steps": len(timed), "gpu_launches": launches, "clocks": clk,
            "last_volume_weighted_global_xH": glob["volume_weighted_global_xH"]}


def run_gb300(args, rank, world, local):
    import torch

    from meraxes_gb300.api import ReionGridStep

    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    init_dist(world, "nccl")
    w = workload_for(args.grid)
    p = w.params
    D = p.grid_dim
    n_snap = len(w.redshifts)
    warm = [i % n_snap for i in range(args.warmup)]
    timed = [i % n_snap for i in range(args.steps)]
    used = sorted(set(warm) | set(timed))
    fields = make_device_fields(w, used, device)

    step = ReionGridStep(p, w.redshifts)
    n_hist = step.n_sfr_histories
    hist, smax = history_buffer(fields, used, n_hist, D, device)
    # the headline: every snapshot's step captured and launched as one CUDA
    # graph; the same evolution uncaptured is timed beside it
    ungraphed = None
    if not args.no_graph:
        ms0, _, _, _, _ = time_evolution(step, w, fields, hist, smax, warm, timed, device, world, local)
        ungraphed = replica_value(ms0, args.steps, world, device)
        step.set_graph(True)
    ms, launches, glob, clk, kstats = time_evolution(step, w, fields, hist, smax, warm, timed, device, world, local,
                                                     profile=True)
    value = replica_value(ms, args.steps, world, device)
    step.set_graph(False)

    # per-kernel achieved bandwidth (algorithmic bytes / event time)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    kernels = {}
    for name, (n, kms, b) in kstats.items():
        kernels[name] = {"launches": n, "ms_per_launch": kms / max(n, 1), "share": kms / max(ms, 1e-9),
                         "gbs": (b / 1e9) / (kms / 1e3) if kms > 0 else None}
    dom = max(kstats.items(), key=lambda kv: kv[1][1]) if kstats else None
    roofline = None
    if dom:
        name, (n, kms, b) = dom
        achieved = (b / n / 1e9) / (kms / n / 1e3)
        ratio = DRAM_PER_ALGORITHMIC.get(name)
        traffic = ratio * b / n if ratio else None
        if traffic and name == "fft_z_threshold":
            traffic += THRESHOLD_STATE_BYTES_PER_CELL * float(D) ** 3
        roofline = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": hbm_peak,
                    "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                    "traffic": round(traffic) if traffic else None,
                    "peak_source": peak_src, "algorithmic_bytes_per_launch": b / n}
    # whole-step algorithmic bandwidth
    total_bytes = sum(v[2] for v in kstats.values())
    step_gbs = (total_bytes / args.steps / 1e9) / (value * world / 1e3)
    # the algorithmic model of a snapshot (every grid read and written once per
    # logical pass, every 3-D FFT one ideal read + write): find_HII_bubbles
    # N (8G + 12 G n_R + 32), ComputeTs N (8 + 12 S + 24), delta_T 16 N
    G = 3 + (1 if p.flag_recombinations else 0) + (1 if p.flag_spin_temp else 0)
    n_R = len(p.filter_radii())
    S = p.ts_num_filter_steps if p.flag_spin_temp else 0
    model_bytes = float(D) ** 3 * ((8 * G + 12 * G * n_R + 32) + ((8 + 12 * S + 24) if S else 0) + 16)
    model_gbs = (model_bytes / 1e9) / (value * world / 1e3)

    # ------------------------------------------------------------------ e2e
    e2e = None
    if not args.no_e2e and args.e2e_steps > 0:
        e2e = run_e2e(args, step, w, fields, hist, smax, timed, n_hist, device, world)
    block_sizes = list(step.fft_block_sizes())
    zpass_blocks = step.zpass_blocks()
    step.close()
    plain = None
    if not args.no_plain:
        plain = run_plain_gpu(args, w, fields, hist, smax, warm, timed, device, world, local)

    del fields, hist
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(value * world, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 grids/FFTs, f64 tables and reductions",
        "data": "synthetic (seeded Gaussian density, stellar and SFR grids)",
        "config": {"workload": f"evolve_512: {D}^3, L={p.box_size} Mpc/h, 20 snapshots z=15..6, "
                               "ComputeTs 40 shells + find_HII_bubbles 41 radii x 5 fields + 21cm box",
                   "grid": D, "snapshots_warmup": warm, "snapshots_timed": timed,
                   "state": "the timed snapshots are one evolution from the initial state (reset after the "
                            "warm-up)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (each grid 0.54 GB at 512^3)",
                   "fft_block_sizes": block_sizes, "zpass_blocks_per_sm": zpass_blocks,
                   "step_graph": not args.no_graph},
        "value_uncaptured": round(ungraphed, 3) if ungraphed is not None else None,
        "gpu_launches": launches, "clocks": clk, "roofline": roofline,
        "step_model_gbs": round(model_gbs, 1), "step_model_frac": round(model_gbs / hbm_peak, 4),
        "step_model_bytes": model_bytes, "step_pass_gbs": round(step_gbs, 1),
        "kernels": {k: {kk: (round(vv, 4) if isinstance(vv, float) else vv) for kk, vv in v.items()}
                    for k, v in kernels.items()},
        "last_globals": {k: glob[k] for k in ("volume_weighted_global_xH", "volume_ave_TS", "volume_ave_Tb")},
    }
    if e2e:
        out["e2e"] = e2e
    if plain:
        plain["ratio_to_value"] = round(plain["value"] / value, 3)
        out["plain_gpu"] = plain
    # the legs beside the headline run in child processes of their own, each
    # with a fresh CUDA context and the device memory to itself; a leg that
    # fails is reported as such and the line is still printed
    if not args.no_adjoint and args.adjoint_grid > 0:
        out["adjoint"] = run_leg(f"bench.run_adjoint_ratio(bench.parse_args(['--adjoint-grid', '{args.adjoint_grid}']))")
    if not args.no_batch and world == 1:
        if args.batch_adjoint:
            out["batch"] = run_leg("bench.run_batch()")
        out["batch_native"] = run_leg("bench.run_batch_native()")
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(args)
    return out, rank


def run_leg(call: str, timeout: float = 1800) -> dict:
    """Runs `call` (an expression over this module) in a child process and
    returns its JSON result, or {"error": ...} if the child failed."""
    code = (f"import sys, json; sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'tests')!r});"
            f"import bench; print(json.dumps({call}))")
    try:
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=timeout)
    except subprocess.TimeoutExpired:
        return {"error": f"timed out after {timeout:.0f} s"}
    if r.returncode != 0:
        return {"error": (r.stderr.strip().splitlines() or ["exit code %d" % r.returncode])[-1][-300:]}
    return json.loads(r.stdout.strip().splitlines()[-1])


def run_adjoint_ratio(args, steps: int = 3):
    """Forward and forward + adjoint of the power-spectrum loss on the
    differentiation workload (diff_256: 256^3, L=100 Mpc/h, seed 3, z=12; the
    20-bin loss against a target made at L_X = 2e40).  Forward: ComputeTs ->
    find_HII_bubbles -> 21cm box -> loss; adjoint: the loss gradient, the
    recomputed shells, the per-cell adjoint and the shell adjoint.  CUDA-event
    times per step, after one warm-up."""
    import numpy as np
    import torch

    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import ReionGridStep
    from meraxes_gb300.autograd import DeltaT21, PSLoss21, log_bins
    from meraxes_gb300.params import workload

    w = workload("diff_256", args.adjoint_grid)
    p = w.params
    step = ReionGridStep(p, w.redshifts)
    gen = syn.FieldGenerator(w)
    st = syn.initial_state(p, w.redshifts[0])
    st.update(gen.inputs(1, step.n_sfr_histories))
    D = p.grid_dim
    st.setdefault("delta_T", np.zeros((D, D, D), np.float32))
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in st.items()}
    state = {k: v for k, v in dev.items() if k not in ("sfr", "stars")}
    edges = log_bins(step, 20)
    lx0 = torch.tensor(p.lx_gal, dtype=torch.float64)
    e00 = torch.tensor(p.nu_xray_gal_threshold, dtype=torch.float64)
    with torch.no_grad():
        dT = DeltaT21.apply(dev["sfr"], dev["stars"], torch.tensor(2e40, dtype=torch.float64), e00, step, 1, state)
        _, target, _ = step.ps_loss(dT, edges, [0.0] * 20, grad=False)
    fwd, tot = [], []
    for i in range(steps + 1):
        sfr = dev["sfr"].clone().requires_grad_(True)
        stars = dev["stars"].clone().requires_grad_(True)
        lx = lx0.clone().requires_grad_(True)
        e0 = e00.clone().requires_grad_(True)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        ev[0].record()
        L = PSLoss21.apply(DeltaT21.apply(sfr, stars, lx, e0, step, 1, state), step, edges, target)
        ev[1].record()
        L.backward()
        ev[2].record()
        torch.cuda.synchronize()
        if i > 0:
            fwd.append(ev[0].elapsed_time(ev[1]))
            tot.append(ev[0].elapsed_time(ev[2]))
    f, t = sum(fwd) / len(fwd), sum(tot) / len(tot)
    del step
    return {"config": f"diff_256: {D}^3, L={p.box_size} Mpc/h, seed 3, z=12, 20-bin power-spectrum loss, "
                      "gradients w.r.t. sfr, stars (escape fraction), L_X, E0",
            "fwd_ms": round(f, 3), "fwd_adj_ms": round(t, 3), "ratio": round(t / f, 3), "steps": steps}


def run_batch():
    """The uneven batch: 48 independent boxes (16 each at 96^3, 128^3, 192^3,
    0.5 Mpc/h cells, seeds 10-57, L_X and escape fraction drawn per box), the
    forward step and the adjoint of the power-spectrum loss for every box, on
    concurrent workers (meraxes_gb300/batch.py).  Wall time of the 48 boxes;
    inputs and loss targets are prepared before it."""
    from meraxes_gb300.batch import BatchRunner, uneven_batch

    runner = BatchRunner(uneven_batch())
    plan = runner.make_plan()
    out = runner.run()
    return {"config": "48 boxes: 16 each at 96^3, 128^3, 192^3, 0.5 Mpc/h cells, forward + adjoint per box",
            "wall_s": round(out["wall_s"], 3), "boxes_per_s": round(48 / out["wall_s"], 2),
            "workers_per_size": {str(k): v for k, v in plan.items()}}


def run_batch_native():
    """The same 48 boxes, forward step only, through the native executor
    mx_batch_run (12 worker threads, each with its own contexts and stream):
    host grids in pinned memory, the escape fraction applied to the stars grid
    as in the differentiable forward.  A first run creates the workers'
    contexts; the timed second run steps every box again on the state the
    first left, with every box's host<->device copies inside the timing."""
    import dataclasses

    import torch

    from meraxes_gb300 import synthetic as syn
    from meraxes_gb300.api import Batch, ReionGridStep
    from meraxes_gb300.batch import instance_workload, uneven_batch

    insts = uneven_batch()
    n_hist = {}
    items = []
    for inst in insts:
        w = instance_workload(inst)
        D = inst.grid_dim
        if D not in n_hist:
            n_hist[D] = ReionGridStep(w.params, w.redshifts, max_work_bytes=25 * 8 * D * D * (D // 2 + 16)).n_sfr_histories
        st = syn.initial_state(w.params, w.redshifts[0])
        st.update(syn.FieldGenerator(w).inputs(1, n_hist[D]))
        st["stars"] = st["stars"] * np.float32(inst.fesc)
        st.setdefault("delta_T", np.zeros((D, D, D), np.float32))
        grids = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory().numpy() for k, v in st.items()}
        items.append({"params": dataclasses.replace(w.params, lx_gal=inst.lx_gal), "redshifts": w.redshifts,
                      "snapshot": 1, "grids": grids})
    batch = Batch(max_workers=12)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch.run(items)  # creates the workers' contexts
    first = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch.run(items)  # the next step of every box, contexts reused
    wall = time.perf_counter() - t0
    # the same 48 boxes as one CUDA graph, launched once (mx_batch_run_graph):
    # a first run creates a context per box, the timed second run captures,
    # instantiates and launches the batch graph
    t0 = time.perf_counter()
    batch.run(items, graph=True)
    gfirst = time.perf_counter() - t0
    t0 = time.perf_counter()
    batch.run(items, graph=True)
    gwall = time.perf_counter() - t0
    batch.close()
    return {"config": "48 boxes: 16 each at 96^3, 128^3, 192^3, 0.5 Mpc/h cells, forward step per box "
                      "(host grids in pinned memory, copies included)",
            "wall_s": round(wall, 3), "boxes_per_s": round(48 / wall, 2), "workers": 12,
            "first_run_s_with_context_creation": round(first, 3),
            "one_launch": {"entry_point": "mx_batch_run_graph (every box in one CUDA graph launch)",
                           "wall_s": round(gwall, 3), "boxes_per_s": round(48 / gwall, 2),
                           "first_run_s_with_context_creation": round(gfirst, 3)}}


def run_e2e(args, step, w, fields, hist, smax, timed, n_hist, device, world):
    """Same metric through the host-pointer entry points, on the same
    evolution as `value`: the timed snapshots from the initial state, every
    snapshot's inputs, state and SFR-history slices in pinned host buffers.
    Each timed call copies its inputs host->device and all outputs back;
    filling the pinned buffers with the next snapshot's inputs is not timed.
    Two legs: mx_step (one call per snapshot), and the reference's three
    entry points called one after another as the C adapter calls them
    (mx_ComputeTs, mx_find_HII_bubbles, mx_ComputeBrightnessTemperatureBox,
    each copying the grids it reads and writes)."""
    import torch

    p = w.params
    D = p.grid_dim
    snaps = timed[: max(1, min(args.e2e_steps, len(timed)))]
    host = {k: v.cpu().pin_memory().numpy() for k, v in fields[snaps[0]].items()}
    st0 = state_grids(p, w.redshifts[0], "cpu")
    for k, v in st0.items():
        host[k] = v.pin_memory().numpy()
    hbuf = None
    if n_hist > 0:
        hbuf = torch.zeros((n_hist, D * D * 2 * (D // 2 + 1)), dtype=torch.float32).pin_memory()
        host["sfr_histories"] = hbuf.numpy()
    # mx_step uploads each input once; x_e_box is not uploaded when ComputeTs
    # runs (it writes x_e_box on the device before find_HII_bubbles reads it)
    in_names = ["deltax", "stars", "weighted_sfr", "N_rec", "z_at_ionization", "J_21_at_ionization",
                "Gamma12", "sfr", "x_e_box_prev", "Tk_box"]
    if not p.flag_spin_temp:
        in_names.append("x_e_box")
    out_names = ["N_rec", "xH", "z_at_ionization", "r_bubble", "J_21", "J_21_at_ionization", "Gamma12", "sfr",
                 "x_e_box", "x_e_box_prev", "Tk_box", "TS_box", "delta_T"]
    nb = lambda n: host[n].nbytes  # noqa: E731
    h2d = sum(nb(n) for n in in_names if n in host) + (host["sfr_histories"].nbytes if n_hist > 0 else 0)
    d2h = sum(nb(n) for n in out_names if n in host)

    def prepare(s):
        for k, v in fields[s].items():
            torch.from_numpy(host[k]).copy_(v.reshape(host[k].shape))
        if hbuf is not None:
            hbuf.copy_(hist[smax - s: smax - s + n_hist])
        torch.cuda.synchronize()

    def reset_state():
        for k, v in st0.items():
            np.copyto(host[k], v.numpy())

    def leg(call):
        reset_state()
        prepare(snaps[0])
        call(snaps[0])  # first host calls allocate the device mirror
        reset_state()
        torch.cuda.synchronize()
        barrier(world)
        t = 0.0
        for s in snaps:
            if s == 0:
                reset_state()
            prepare(s)
            t0 = time.perf_counter()
            call(s)
            t += time.perf_counter() - t0
        return replica_value(t * 1e3, len(snaps), world, device)

    def three(s):
        step.ComputeTs(s, host)
        step.find_HII_bubbles(s, host)
        step.ComputeBrightnessTemperatureBox(s, host)

    v1 = leg(lambda s: step.step(s, host))
    v3 = leg(three)
    return {"value": round(v1, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "steps": len(snaps), "snapshots": snaps, "entry_point": "mx_step (host pointers)",
            "three_calls": {"value": round(v3, 3), "unit": UNIT,
                            "entry_points": "mx_ComputeTs, mx_find_HII_bubbles, "
                                            "mx_ComputeBrightnessTemperatureBox (host pointers, as the C "
                                            "adapter calls them)"}}


# CPU timing.  The reference runs this step on CPU cores (FFTW float
# transforms, per-cell C loops); its CPU path is timed here as the oracle
# port built with single-precision transforms (oracle/_build/
# libmxoracle_f32.so: batched Stockham FFTs and per-cell loops on all host
# threads) at the benchmark's own grid size.  A full 512^3 snapshot takes
# minutes, so a timed snapshot is a bounded sample of itself: the first
# `radii` radii of find_HII_bubbles, the first `shells` ComputeTs shells and
# 1/`cell_div` of the per-cell spin-temperature work are run and timed, and
# the per-radius, per-shell and per-cell times are scaled to the workload's 41
# radii, 40 shells and all cells.  Everything else (the forward transforms,
# the collapse fraction, the frequency-integral tables, the global means,
# N_rec, delta_T) runs in full.  The oracle keeps its grid buffers across
# calls, as the reference allocates its grids once, so the first snapshot of
# a process also pays the first touch of those buffers and is not timed.
CPU_SAMPLE = {"radii": 3, "shells": 3, "cell_div": 16}
# per step of the reference arm, which runs W + K sampled snapshots
REF_SAMPLE = {"radii": 2, "shells": 2, "cell_div": 64}


def cpu_run(grid: int, threads: int, radii: int, shells: int, cell_div: int, runs: int) -> dict:
    """Runs `runs` sampled snapshots (snapshot 10 of evolve_512 at grid^3) of
    the oracle port in this process; returns each run's estimated full
    snapshot time (s) with its measured parts."""
    from meraxes_gb300 import synthetic as syn
    from oracle import OracleBackend

    w = workload_for(grid)
    n_R = len(w.params.filter_radii())
    S = w.params.ts_num_filter_steps
    orc = OracleBackend(w.params, w.redshifts, syn.TABLES_DIR, timing=True)
    orc.set_timing_sample(radii, shells, cell_div)
    gen = syn.FieldGenerator(w)
    s = 10
    st0 = syn.initial_state(w.params, w.redshifts[s - 1])
    st0.update(gen.inputs(s, orc.n_sfr_histories))
    out = []
    for _ in range(runs):
        st = {k: v.copy() for k, v in st0.items()}
        t0 = time.perf_counter()
        orc.ComputeTs(s, st)
        t1 = time.perf_counter()
        ts = orc.phase_times()
        orc.find_HII_bubbles(s, st)
        t2 = time.perf_counter()
        fh = orc.phase_times()
        orc.delta_T(s, st)
        t3 = time.perf_counter()
        per_radius = fh["radii"] / max(fh["n_radii"], 1)
        per_shell = ts["shells"] / max(ts["n_shells"], 1)
        est_ts = (t1 - t0) - ts["shell_copies"] + per_shell * (S - ts["n_shells_run"]) \
            + ts["evolve"] * (1.0 / ts["evolve_frac"] - 1.0)
        est_fhb = (t2 - t1) + per_radius * (n_R - fh["n_radii_run"])
        out.append({"estimate_s": est_ts + est_fhb + (t3 - t2), "sampled_s": t3 - t0, "ComputeTs_s": est_ts,
                    "find_HII_bubbles_s": est_fhb, "delta_T_s": t3 - t2, "per_radius_s": per_radius,
                    "per_shell_s": per_shell, "evolve_s": ts["evolve"] / ts["evolve_frac"],
                    "forward_s": fh["forward"], "tables_s": ts["tables"]})
    orc.close()
    return {"grid": grid, "threads": threads, "n_radii": n_R, "n_shells": S, "runs": out}


def cpu_runs(grid: int, threads: int, runs: int, sample=None, timeout: float = 3000) -> dict:
    """cpu_run in a child process with OMP_NUM_THREADS = threads (the child
    keeps the oracle's OpenMP pool away from this process's CUDA context)."""
    smp = dict(CPU_SAMPLE if sample is None else sample)
    smp["cell_div"] = min(smp["cell_div"], grid)  # at least one x plane of cells
    code = (f"import sys, json; sys.path.insert(0, {ROOT!r}); sys.path.insert(0, {os.path.join(ROOT, 'tests')!r});"
            f"import bench; print(json.dumps(bench.cpu_run({grid}, {threads}, {smp['radii']}, {smp['shells']}, "
            f"{smp['cell_div']}, {runs})))")
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="false")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-500:])
    res = json.loads(r.stdout.strip().splitlines()[-1])
    res["sample"] = smp
    return res


def cpu_sample_text(res: dict, timed: list) -> str:
    smp = res["sample"]
    r = timed[-1]
    return (f"oracle port with single-precision transforms (oracle/_build/libmxoracle_f32.so), {res['threads']} "
            f"host threads, snapshot 10 of evolve_512 at {res['grid']}^3; each timed snapshot runs the forward "
            f"transforms, tables, means, N_rec and delta_T in full and {smp['radii']} of {res['n_radii']} radii, "
            f"{smp['shells']} of {res['n_shells']} shells and 1/{smp['cell_div']} of the per-cell spin-temperature "
            f"work, timed and scaled to the full counts (measured at {res['grid']}^3: {r['per_radius_s']:.2f} s per "
            f"radius, {r['per_shell_s']:.2f} s per shell, {r['evolve_s']:.1f} s per-cell evolution, "
            f"{r['forward_s']:.2f} s forward transforms; {r['sampled_s']:.1f} s of CPU work per timed snapshot); "
            f"one untimed snapshot first")


def cpu_baseline(args):
    threads = os.cpu_count() or 1
    try:
        res = cpu_runs(args.grid, threads, 2)
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": UNIT, "error": str(e)[-300:]}
    timed = res["runs"][1:]
    est = timed[-1]["estimate_s"]
    return {"value": round(est * 1e3, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": cpu_sample_text(res, timed),
            "parts_s": {k: round(v, 3) for k, v in timed[-1].items()}}


def run_reference(args, rank, world):
    """The CPU implementation of the path on all host threads: the oracle
    port (the reference's own build needs FFTW/GSL/MPI/HDF5 and the reference
    tree, absent on the GPU host), each step one sampled snapshot at the
    benchmark's grid size (REF_SAMPLE), after W warm-up snapshots."""
    if rank != 0:
        return None, rank
    threads = os.cpu_count() or 1
    try:
        res = cpu_runs(args.grid, threads, max(args.warmup, 1) + args.steps, sample=REF_SAMPLE)
    except Exception as e:  # noqa: BLE001
        return {"impl": "reference", "unavailable": "oracle port failed: " + str(e)[-300:]}, rank
    timed = res["runs"][max(args.warmup, 1):]
    value = statistics.mean(r["estimate_s"] for r in timed) * 1e3
    sample = cpu_sample_text(res, timed)
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(value, 1), "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 grids and transforms, f64 physics",
            "data": "synthetic", "config": {"workload": f"evolve_512 at {args.grid}^3 (sampled snapshots)"},
            "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "steps_s": [round(r["estimate_s"], 2) for r in timed]}, rank


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out, rank = run_reference(args, rank, world)
    else:
        out, rank = run_gb300(args, rank, world, local)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
