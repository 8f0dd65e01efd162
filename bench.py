#!/usr/bin/env python3
"""Throughput of the w-stacking hot path: Mvis/s for forward + adjoint imaging.

Workload (the precision configuration): a 4096 x 4096 grid, 32 w-planes,
support 7, 50,000,000 visibilities from 62 stations in an 8 km disk observed
for 8 h at 150 MHz (seeded synthetic data: stations, earth-rotation uvw
tracks, 20 point sources + noise).  One step = forward imaging (bin + grid +
per-plane inverse FFT + w-correction) followed by the adjoint (w-correction
adjoint + per-plane forward FFT + degridding), in the FP32-compensated form.
Inputs (1.8 GB) and the grid (4.3 GB) exceed L2 (129 MB), so no L2 flush.

Also reported on the same inputs: the plain FP64 form (its Mvis/s and the
FP32C/FP64 dirty-image error), the end-to-end figure through the C ABI with
host buffers, per-stage CUDA-event times with the HBM roofline of each stage,
and the reference's OpenMP CPU path (the oracle port) timed on a bounded
sample on this host's cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
    python bench.py --workload c4     # the (channel, polarisation) batch: 16 channels
                                      # x 4 polarisations, 2048^2 x 16 planes each
    python bench.py --workload driver --steps 3   # the reference's main() on files:
                                      # read a dataset directory, grid, FFT, w-correct,
                                      # write the image dump (wsg_run_paramfile)

Roofline traffic (DRAM bytes per launch of the gridding stage's kernels) is
read from the committed ncu launch-list summary of the same workload
(profiles/launches_fwd_adj_4096x32_50M.md) and scaled by the records binned
when the workload differs.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mvis/s fwd+adjoint, FP32-comp vs FP64 at <=1e-5 rel image err; % HBM roofline"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--layout", default="walk", choices=["walk", "index"],
                    help="walk: the plan is told the measurements' [dump][baseline] layout "
                         "(wsg_plan_set_layout) and bins along tracks; index: binning in "
                         "index order, as for inputs of unknown layout")
    ap.add_argument("--shard", default="replicas", choices=["replicas", "planes"],
                    help="N>1: replicas (every GPU images the whole workload, no exchange) or "
                         "planes (one image; each GPU grids, transforms and w-corrects its "
                         "w-plane range and the partial images are sum-reduced with NCCL)")
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c4", "c5", "driver"],
                    help="c2: one 4096^2 x 32 image (default); c1: the reference's CPU "
                         "configuration (512^2 x 8, 1M visibilities, 48 stations, 3 km, 4 h) "
                         "with the reference CPU path timed in full beside it; "
                         "c4: the channel x pol batch; "
                         "c5: one 8192^2 x 128 image, support 9, 400M visibilities; "
                         "driver: c2 as files through the reference's main()")
    ap.add_argument("--driver-dir", default=None,
                    help="driver: directory for the dataset and dump files (default: a temp dir)")
    ap.add_argument("--driver-write-data", action="store_true",
                    help="driver: also time one run with the grid and fft dumps")
    ap.add_argument("--subset", type=int, default=1_000_000,
                    help="c5: visibilities in the subset checked against the FP64 oracle")
    ap.add_argument("--window", type=int, default=512, help="c5: edge of the checked window")
    ap.add_argument("--per-channel", type=int, default=8_000_000,
                    help="c4: measurements per channel before flagging")
    ap.add_argument("--channels", type=int, default=16)
    ap.add_argument("--nvis", type=int, default=None, help="default: the workload's")
    ap.add_argument("--nx", type=int, default=None)
    ap.add_argument("--planes", type=int, default=None)
    ap.add_argument("--support", type=int, default=None)
    ap.add_argument("--fp64-steps", type=int, default=2)
    # as many as the timed device steps: the first step's upload cannot
    # overlap a previous step, a fill cost spread over the steps
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args()
    from lofar_gb300 import synth
    cfg = synth.CONFIGS[a.workload if a.workload in ("c1", "c5") else "c2"]
    a.nvis = cfg["gen"]["n_vis"] if a.nvis is None else a.nvis
    a.nx = cfg["nx"] if a.nx is None else a.nx
    a.planes = cfg["planes"] if a.planes is None else a.planes
    a.support = cfg["support"] if a.support is None else a.support
    return a


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        try:
            d = json.load(open(path))
            for k in ("hbm_gbs", "hbm_GBps", "hbm"):
                if k in d:
                    return float(d[k]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


# ---------------------------------------------------------------------------
# ranks: replicas only (every rank runs the whole workload on its own GPU;
# the path has no exchange step at one image per rank)
# ---------------------------------------------------------------------------

def max_over_ranks(x: float, world: int) -> float:
    """The slowest rank's time (the job ends when the last rank does)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.barrier()
    return float(t.item())


def whole_job_mvis(n_per_rank: int, world: int, ms_per_step: float) -> float:
    """Visibilities of all ranks per second of the slowest rank, in millions."""
    return n_per_rank * world / (ms_per_step * 1e-3) / 1e6


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def workload(args, backend):
    from lofar_gb300 import synth
    gen = dict(synth.CONFIGS["c1" if args.workload == "c1" else "c2"]["gen"])
    gen["n_vis"] = args.nvis
    t = time.time()
    obs = synth.observe(backend=backend, **gen)
    res = obs.resolution
    return obs, res, time.time() - t


def algorithmic_bytes(n, nx, ny, planes, sc):
    """Per-stage algorithmic bytes (read inputs once, write outputs once).

    The FFT + w-correction stages count one read of the grid and one write of
    the image (and the reverse for the adjoint): the transformed planes are
    an intermediate of the fused kernels."""
    cells = planes * nx * ny
    return {
        "grid": n * (24 + 8 + 4) + cells * sc,          # bin + grid: inputs in, grid out
        "fft_wcorrect": cells * sc + nx * ny * sc,
        "wcorrect_adj_fft": nx * ny * sc + cells * sc,
        "degrid": cells * sc + n * 24 + n * sc,          # grid + uvw in, values out
    }


PROFILE_MD = os.path.join(ROOT, "profiles", "launches_fwd_adj_4096x32_50M.md")
GRIDDING_KERNELS = ("k_bin_count", "k_bin_count_rows", "k_bin_scan_a", "k_bin_scan_b",
                    "k_bin_scan_c", "k_bin_scatter", "k_bin_scatter_rows", "k_fft_masks",
                    "k_grid_f32c")
PROFILE_RECORDS = 59_834_420   # records binned in the profiled run (4096^2 x 32, 50M)


def profiled_traffic(records):
    """DRAM bytes (read + write) per launch of the gridding-stage kernels, from
    the ncu launch list, scaled to `records` records; None if unavailable."""
    if not os.path.exists(PROFILE_MD):
        return None
    tot, seen = 0.0, set()
    for ln in open(PROFILE_MD):
        f = [x.strip().strip("`") for x in ln.split("|")]
        if len(f) < 8 or not f[1].startswith("k_"):
            continue
        name = f[1].split("<")[0]
        if name in GRIDDING_KERNELS:
            try:
                tot += (float(f[5]) + float(f[6])) * 1e9
                seen.add(name)
            except ValueError:
                pass
    if "k_grid_f32c" not in seen or not seen & {"k_bin_scatter", "k_bin_scatter_rows"}:
        return None
    return tot * records / PROFILE_RECORDS


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------

STAGES = ["bin", "grid", "fft_wcorrect", "wcorrect_adj_fft", "degrid"]
# count + scan(3) + scatter + tile masks; grid; column FFT + row FFT/w-correction;
# row FFT/adjoint w-correction + column FFT; degrid
OUR_KERNELS_PER_STEP = {"bin": 6, "grid": 1, "fft_wcorrect": 2, "wcorrect_adj_fft": 2,
                        "degrid": 1}


L2_BYTES = 129 * 1000 * 1000   # GB300 L2


def l2_flush_bytes(working_set):
    """Bytes to write between timed steps so that no step starts with the
    previous step's data in L2: 0 when the step's working set (inputs, grid)
    is over twice the L2, else 256 MB."""
    return 0 if working_set > 2 * L2_BYTES else 256 << 20


def l2_note(flush):
    return ("L2 flushed before every step (256 MB written outside the timed region)" if flush
            else "inputs larger than L2 (no flush)")


def run_plan_steps(plan, ins, image, out, steps, record_stages, reduce=None, flush=0):
    """`steps` forward+adjoint passes; returns (total_ms, {stage: [ms per step]}).
    reduce: applied to the forward image before the adjoint (the plane-sharded
    form's sum over ranks).  flush: bytes written before every step, outside
    the timed region (the total is then the sum of the steps' own times)."""
    import torch
    stream = torch.cuda.current_stream()
    per = {s: [] for s in STAGES}
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    scratch = torch.empty(flush, dtype=torch.uint8, device="cuda") if flush else None
    pending = []
    start.record(stream)
    for _ in range(steps):
        if scratch is not None:
            scratch.zero_()
        evs = ([torch.cuda.Event(enable_timing=True) for _ in range(len(STAGES) + 1)]
               if record_stages or flush else None)
        if evs:
            evs[0].record(stream)
        plan.bin(*ins)
        if evs:
            evs[1].record(stream)
        grid = plan.grid(plan_grid(plan), occupied_only=True)
        if evs:
            evs[2].record(stream)
        plan.fft_wcorrect(grid, out=image)
        if reduce is not None:
            reduce(image)
        if evs:
            evs[3].record(stream)
        plan.wcorrect_adjoint_fft(image, out=grid)
        if evs:
            evs[4].record(stream)
        plan.degrid(grid, out=out)
        if evs:
            evs[5].record(stream)
            pending.append(evs)
    stop.record(stream)
    torch.cuda.synchronize()
    for evs in pending:
        for i, s in enumerate(STAGES):
            per[s].append(evs[i].elapsed_time(evs[i + 1]))
    if flush:
        return sum(evs[0].elapsed_time(evs[-1]) for evs in pending), per
    return start.elapsed_time(stop), per


_GRIDS = {}


def plan_grid(plan):
    key = id(plan)
    if key not in _GRIDS:
        _GRIDS[key] = plan.new_grid()
    return _GRIDS[key]


def bench_ours(args, rank, world):
    import torch
    import torch.distributed as dist
    from lofar_gb300 import Plan

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    obs, res, gen_s = workload(args, "torch")
    n = obs.n
    nx = ny = args.nx
    P = args.planes

    t = torch.cuda
    ins = (torch.as_tensor(obs.uu).cuda(), torch.as_tensor(obs.vv).cuda(),
           torch.as_tensor(obs.ww).cuda(), torch.as_tensor(obs.vis_real).cuda(),
           torch.as_tensor(obs.vis_img).cuda(), torch.as_tensor(obs.weight).cuda())
    reduce = None
    planes_mode = args.shard == "planes" and world > 1
    if planes_mode:
        # one image over all ranks: this rank's w-plane range and measurements;
        # the partial images are summed by NCCL between forward and adjoint
        from lofar_gb300.sharding import PlaneShard, plane_counts
        shard = PlaneShard(P, 1.0 / P, plane_counts(obs.ww, 1.0 / P, P))
        _, ins = shard.select(*ins)
        reduce = shard._all_reduce
    n_local = int(ins[0].numel())

    # the synthetic measurements are [dump][baseline], as the reference's
    # measurement sets are (meta.txt's `baselines`): the binning walks tracks
    rows = 0 if planes_mode or args.layout == "index" else obs.meta.get("n_baselines", 0)
    plan = Plan(nx, ny, P, args.support, precision="fp32c")
    plan.set_wcorrection(res, obs.wmin, obs.wmax)
    plan.set_layout(rows)
    plan.reserve(n_local)
    image = torch.empty((ny, nx), dtype=torch.complex64, device="cuda")
    out = torch.empty(n_local, dtype=torch.complex64, device="cuda")

    # warm-up (also builds the w-screen table and the cuFFT plan)
    run_plan_steps(plan, ins, image, out, args.warmup, False, reduce)
    stats = plan.stats()
    flush = l2_flush_bytes(n_local * 36 + P * nx * ny * 8)

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    total_ms, per = run_plan_steps(plan, ins, image, out, args.steps, True, reduce, flush)
    clk = clocks.stop()
    total_ms = max_over_ranks(total_ms, world)
    ms_per_step = total_ms / args.steps
    # replicas: every rank imaged all n visibilities; planes: one image of n
    value = whole_job_mvis(n, 1 if planes_mode else world, ms_per_step)
    if planes_mode:
        return dict(rank=rank, n=n, res=res, wmin=obs.wmin, wmax=obs.wmax, gen_s=gen_s,
                    ms_per_step=ms_per_step, value=value, per=per, stats=stats, clocks=clk,
                    plan_bytes=plan.device_bytes(), planes=(shard.p0, shard.p1)), obs

    # forward image of the FP32C form (for the accuracy comparison)
    img32 = plan.image_forward(*ins).clone()
    torch.cuda.synchronize()

    result = dict(rank=rank, n=n, res=res, wmin=obs.wmin, wmax=obs.wmax, gen_s=gen_s,
                  ms_per_step=ms_per_step, value=value, per=per, stats=stats, clocks=clk,
                  plan_bytes=plan.device_bytes(), l2=l2_note(flush),
                  layout=(f"[dump][baseline] walk, {rows} rows per dump" if rows
                          else "index order"))

    # -- plain FP64 form, same inputs --------------------------------------
    if not args.no_fp64 and rank == 0:
        del _GRIDS[id(plan)]
        plan.close()
        torch.cuda.empty_cache()
        p64 = Plan(nx, ny, P, args.support, precision="fp64")
        p64.set_wcorrection(res, obs.wmin, obs.wmax)
        p64.reserve(n)
        image64 = torch.empty((ny, nx), dtype=torch.complex128, device="cuda")
        out64 = torch.empty(n, dtype=torch.complex128, device="cuda")
        run_plan_steps(p64, ins, image64, out64, 1, False)
        ms64, per64 = run_plan_steps(p64, ins, image64, out64, args.fp64_steps, True,
                                     flush=l2_flush_bytes(n * 36 + P * nx * ny * 16))
        img64 = p64.image_forward(*ins)
        torch.cuda.synchronize()
        a = torch.view_as_real(img32).double()
        b = torch.view_as_real(img64)
        fin = torch.isfinite(b[..., 0])
        nan_equal = bool(torch.equal(torch.isnan(a[..., 0]), torch.isnan(b[..., 0])))
        diff = (a - b)[fin]
        err_rms = float(torch.sqrt((diff ** 2).mean() / (b[fin] ** 2).mean()).item())
        err_max = float((diff.abs().max() / b[fin].abs().max()).item())
        # per-plane grid error (FP32C grid vs FP64 grid) on the same binning
        plan32 = Plan(nx, ny, P, args.support, precision="fp32c")
        plan32.bin(*ins)
        g32 = plan32.grid()
        p64.bin(*ins)
        g64 = p64.grid(plan_grid(p64))
        plane_err = []
        for w in range(P):
            d = torch.view_as_real(g32[w]).double() - torch.view_as_real(g64[w])
            den = torch.sqrt((torch.view_as_real(g64[w]) ** 2).mean())
            plane_err.append(float((torch.sqrt((d ** 2).mean()) / den).item()) if den > 0 else 0.0)
        result["fp64"] = dict(ms_per_step=ms64 / args.fp64_steps,
                              value=n / (ms64 / args.fp64_steps * 1e-3) / 1e6, per=per64,
                              image_rel_rms=err_rms, image_rel_max=err_max, nan_mask_equal=nan_equal,
                              plane_rel_rms_max=max(plane_err), plane_rel_rms=plane_err)
        plan32.close()
        del _GRIDS[id(p64)]
        p64.close()
        del img64, g64, g32, image64, out64
        torch.cuda.empty_cache()
    else:
        if id(plan) in _GRIDS:
            del _GRIDS[id(plan)]
        plan.close()
        torch.cuda.empty_cache()

    # -- end to end through the C ABI with host buffers ---------------------
    if rank == 0 and args.e2e_steps > 0:
        pin = {k: torch.as_tensor(getattr(obs, k)).pin_memory()
               for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight")}
        himg = torch.empty((ny, nx), dtype=torch.complex64).pin_memory()
        hout = torch.empty(n, dtype=torch.complex64).pin_memory()
        pe = Plan(nx, ny, P, args.support, precision="fp32c")
        pe.set_wcorrection(res, obs.wmin, obs.wmax)
        pe.set_layout(rows)
        args_h = [pin[k] for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight")]
        pe.image_forward_host(*args_h, himg)
        pe.image_adjoint_host(himg, hout)
        torch.cuda.synchronize()
        # blocking calls: every copy and kernel of a step in sequence
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            pe.image_forward_host(*args_h, himg)
            pe.image_adjoint_host(himg, hout)
        blocking_s = (time.perf_counter() - t0) / args.e2e_steps
        # the same steps through the asynchronous calls: a step's uploads
        # overlap the previous step's kernels, its downloads the next step's
        pe.image_forward_host_async(*args_h, himg)
        pe.image_adjoint_host_async(himg, hout)
        pe.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            pe.image_forward_host_async(*args_h, himg)
            pe.image_adjoint_host_async(himg, hout)
        pe.synchronize()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        h2d = sum(int(x.numel() * x.element_size()) for x in args_h) + himg.numel() * 8
        d2h = himg.numel() * 8 + hout.numel() * 8
        result["e2e"] = dict(value=n / e2e_s / 1e6, unit="Mvis/s", h2d_bytes_per_step=int(h2d),
                             d2h_bytes_per_step=int(d2h), ms_per_step=e2e_s * 1e3,
                             steps=args.e2e_steps,
                             api="wsg_image_forward_host_async + wsg_image_adjoint_host_async, "
                                 "pinned host buffers, one wsg_plan_synchronize after the steps",
                             blocking=dict(value=n / blocking_s / 1e6, ms_per_step=blocking_s * 1e3,
                                           api="wsg_image_forward_host + wsg_image_adjoint_host"))
        pe.close()
    return result, obs


# ---------------------------------------------------------------------------
# CPU baseline: the reference's OpenMP path (oracle port), bounded sample
# ---------------------------------------------------------------------------

def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_step(obs, res, args, cores, grid):
    """One whole fwd+adjoint step of the reference's CPU algorithm (the oracle
    port, OpenMP on `cores` threads) on every measurement and every plane:
    wstack (w-stacking.cu:222-311), the per-plane FFTW_BACKWARD x 1/(Nx*Ny)
    (fourier_transform.c:25-59; scipy.fft stands in for FFTW, which is not
    installed), phase_correction (phase_correction.cu:147-207), then the
    adjoint chain (w-correction adjoint, forward FFT x 1/(Nx*Ny), degridding).
    grid: a preallocated float64 [P][ny][nx][2] buffer.  Returns the seconds
    of each stage."""
    import scipy.fft as sfft
    from oracle import oracle as O
    nx = ny = args.nx
    P = args.planes
    kw = dict(num_w_planes=P, dx=1 / nx, dw=1 / P, w_support=args.support, nx=nx, ny=ny)
    wc = dict(nx=nx, ny=ny, num_w_planes=P, resolution=res, wmin=obs.wmin, wmax=obs.wmax,
              num_threads=cores)
    t = {}
    c = time.perf_counter()

    def lap(name):
        nonlocal c
        now = time.perf_counter()
        t[name] = now - c
        c = now

    def fft_in_place(buf, forward):
        z = buf.view(np.complex128)[..., 0]
        f = sfft.fft2 if forward else sfft.ifft2
        r = f(z, axes=(-2, -1), workers=cores, overwrite_x=True)
        if forward:
            r /= float(nx) * float(ny)
        if not np.shares_memory(r, z):
            z[...] = r

    grid[...] = 0.0
    O.wstack(obs.uu, obs.vv, obs.ww, obs.vis_real, obs.vis_img, obs.weight,
             num_threads=cores, grid=grid, **kw)
    lap("grid")
    fft_in_place(grid, forward=False)
    lap("fft")
    re, im = O.phase_correction(grid, **wc)
    lap("wcorrect")
    # the adjoint of the image just formed (pixels where the reference's
    # w-correction is undefined excluded)
    planes = O.phase_adjoint(np.nan_to_num(re), np.nan_to_num(im), **wc)
    lap("wcorrect_adj")
    fft_in_place(planes, forward=True)
    lap("fft_adj")
    O.degrid(obs.uu, obs.vv, obs.ww, planes, num_threads=cores, **kw)
    lap("degrid")
    return t


def cpu_baseline(obs, res, args, steps=1):
    """The reference's CPU path timed over whole steps of the same workload on
    this host's cores (no sampling, no extrapolation)."""
    cores = cpu_cores()
    grid = np.zeros((args.planes, args.nx, args.nx, 2), np.float64)   # touched once, reused
    per = [reference_step(obs, res, args, cores, grid) for _ in range(steps)]
    tot = [sum(p.values()) for p in per]
    step_s = statistics.median(tot)
    return dict(value=obs.n / step_s / 1e6, unit="Mvis/s", cores=cores, kind="port",
                sample=(f"oracle port (OpenMP, {cores} threads; scipy.fft as the FFTW "
                        f"substitute): {steps} whole fwd+adjoint step(s) over all {obs.n} "
                        f"measurements and all {args.planes} planes of the "
                        f"{args.nx}x{args.nx} grid"),
                seconds_per_step=step_s,
                stages_s={k: statistics.median(p[k] for p in per) for k in per[0]})


def bench_reference(args, rank, world):
    """--impl reference: the reference's CPU path (oracle port) on this host,
    whole steps of the same workload (one untimed warm-up step: the buffers and
    the FFT plans are first touched there)."""
    if rank != 0:
        return None
    obs, res, _ = workload(args, "numpy")
    from oracle import build as obuild
    obuild.build_oracle()
    cores = cpu_cores()
    grid = np.zeros((args.planes, args.nx, args.nx, 2), np.float64)
    for _ in range(min(args.warmup, 1)):
        reference_step(obs, res, args, cores, grid)
    t0 = time.perf_counter()
    per = [reference_step(obs, res, args, cores, grid) for _ in range(args.steps)]
    wall = time.perf_counter() - t0
    step_s = wall / max(args.steps, 1)
    value = obs.n / step_s / 1e6
    cb = dict(value=value, unit="Mvis/s", cores=cores, kind="port",
              sample=(f"oracle port (OpenMP, {cores} threads; scipy.fft as the FFTW "
                      f"substitute): {args.steps} timed whole fwd+adjoint steps over all "
                      f"{obs.n} measurements and {args.planes} planes, after "
                      f"{min(args.warmup, 1)} untimed"),
              seconds_per_step=step_s,
              stages_s={k: statistics.median(p[k] for p in per) for k in per[0]})
    return {
        "metric": METRIC, "value": value, "unit": "Mvis/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": (f"synthetic (seeded; {obs.meta['n_stations']} stations, "
                 f"{obs.meta['diameter_m'] / 1000:g} km, {obs.meta['hours']:g} h)"),
        "config": {"workload": f"w-stacking fwd+adjoint, {args.nx}x{args.nx} grid, {args.planes} "
                               f"w-planes, support {args.support}, {obs.n} visibilities",
                   "parallelism": f"replicas{args.gpus}", "l2": "inputs larger than L2"},
        "impl": "reference", "cpu_baseline": cb,
        "e2e": {"value": value, "unit": "Mvis/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }


# ---------------------------------------------------------------------------
# the (channel, polarisation) batch
# ---------------------------------------------------------------------------

def batch_workload(args, backend):
    from lofar_gb300 import synth
    gen = dict(synth.CONFIGS["c4"]["gen"])
    gen["n_per_channel"] = args.per_channel
    gen["n_channels"] = args.channels
    t = time.time()
    obs = synth.observe_batch(backend=backend, **gen)
    return obs, time.time() - t


def bench_batch(args, rank, world, peak, peak_kind):
    """All channel x pol jobs in one persistent gridding launch, the forward
    replayed as one CUDA graph, tuning picked by the autotuner; beside it the
    same jobs run one after another through the single-image plan."""
    import torch
    import torch.distributed as dist
    from lofar_gb300 import Batch, Plan, synth

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    cfg = synth.CONFIGS["c4"]
    nx, P, S = cfg["nx"], cfg["planes"], cfg["support"]
    obs, gen_s = batch_workload(args, "torch")
    C, pols = len(obs.channels), obs.pols
    B = Batch(nx, nx, P, S, channels=C, pols=pols)
    B.set_wcorrection(obs.resolution, obs.wmin, obs.wmax)
    B.bind(obs.channels)
    nvis = B.n_vis()
    images = B.new_images()
    out = torch.empty(nvis, dtype=torch.complex64, device="cuda")
    best, tried = B.autotune(images, iters=2)
    for _ in range(max(args.warmup, 1)):
        B.forward(images, graph=True)
        B.adjoint(images, out)
    stats = B.stats()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    evs = []
    clocks = ClockSampler(dev)
    clocks.start()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(args.steps):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record(stream)
        B.forward(images, graph=True)
        e[1].record(stream)
        B.adjoint(images, out)
        e[2].record(stream)
        evs.append(e)
    stop.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = max_over_ranks(start.elapsed_time(stop), world)
    ms = total_ms / args.steps
    fwd = statistics.median(e[0].elapsed_time(e[1]) for e in evs)
    adj = statistics.median(e[1].elapsed_time(e[2]) for e in evs)
    if rank != 0:
        return None

    # end to end: pinned host inputs -> bound device buffers, forward + adjoint,
    # images and model visibilities back to pinned host memory
    host_in = [[torch.as_tensor(x).pin_memory() for x in ch] for ch in obs.channels]
    himg = torch.empty(images.shape, dtype=torch.complex64).pin_memory()
    hout = torch.empty(nvis, dtype=torch.complex64).pin_memory()

    def e2e_step():
        for dst, src in zip(B._bound, host_in):
            for d, h in zip(dst, src):
                d.copy_(h, non_blocking=True)
        B.forward(images, graph=True)
        B.adjoint(images, out)
        himg.copy_(images, non_blocking=True)
        hout.copy_(out, non_blocking=True)
        torch.cuda.synchronize()

    e2e_step()
    t0 = time.perf_counter()
    n_e2e = max(args.e2e_steps, 1)
    for _ in range(n_e2e):
        e2e_step()
    blocking_s = (time.perf_counter() - t0) / n_e2e

    # the same steps pipelined over three streams: a step's inputs are uploaded
    # while the previous step's adjoint runs (the forward has binned the bound
    # inputs by then), its images and model visibilities are downloaded while
    # the next kernels run
    comp = torch.cuda.current_stream()
    copy_s, out_s = torch.cuda.Stream(), torch.cuda.Stream()

    def upload():
        with torch.cuda.stream(copy_s):
            for dst, src in zip(B._bound, host_in):
                for d, h in zip(dst, src):
                    d.copy_(h, non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(copy_s)
        return ev

    def pipelined(k):
        ev_in = upload()
        ev_img = ev_vis = None
        for i in range(k):
            comp.wait_event(ev_in)
            if ev_img is not None:
                comp.wait_event(ev_img)   # the previous images have left the device buffer
            B.forward(images, graph=True)
            ev_fwd = torch.cuda.Event()
            ev_fwd.record(comp)
            if i + 1 < k:
                copy_s.wait_event(ev_fwd)
                ev_in = upload()
            out_s.wait_event(ev_fwd)
            with torch.cuda.stream(out_s):
                himg.copy_(images, non_blocking=True)
            ev_img = torch.cuda.Event()
            ev_img.record(out_s)
            if ev_vis is not None:
                comp.wait_event(ev_vis)
            B.adjoint(images, out)
            ev_adj = torch.cuda.Event()
            ev_adj.record(comp)
            out_s.wait_event(ev_adj)
            with torch.cuda.stream(out_s):
                hout.copy_(out, non_blocking=True)
            ev_vis = torch.cuda.Event()
            ev_vis.record(out_s)
        torch.cuda.synchronize()

    pipelined(1)
    t0 = time.perf_counter()
    pipelined(n_e2e)
    e2e_s = (time.perf_counter() - t0) / n_e2e
    h2d = sum(int(h.numel() * h.element_size()) for ch in host_in for h in ch)
    d2h = int(himg.numel() * 8 + hout.numel() * 8)

    # the same jobs one after another through the single-image plan
    pl = Plan(nx, nx, P, S, precision="fp32c")
    pl.set_wcorrection(obs.resolution, obs.wmin, obs.wmax)
    jobs = []
    for c, ch in enumerate(B._bound):
        for p in range(pols):
            if ch[0].numel():
                jobs.append((c, p, (ch[0], ch[1], ch[2], ch[3][p::pols].contiguous(),
                                    ch[4][p::pols].contiguous(), ch[5][p::pols].contiguous())))
    img1 = torch.empty((nx, nx), dtype=torch.complex64, device="cuda")
    pl.reserve(max(j[2][0].numel() for j in jobs))

    def seq_step():
        for c, p, ins in jobs:
            pl.image_forward(*ins, out=img1)
            pl.image_adjoint(img1)

    seq_step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_step()
    torch.cuda.synchronize()
    seq_ms = (time.perf_counter() - t0) * 1e3
    pl.close()

    cells = C * pols * P * nx * nx
    ab = algorithmic_bytes(nvis, nx, nx, C * pols * P, 8)
    # per job the image is nx*nx: the cube-wide formula counts one image, add the rest
    ab_step = sum(ab.values()) + 2 * (C * pols - 1) * nx * nx * 8
    gbs = ab_step / (ms * 1e-3) / 1e9
    return {
        "metric": METRIC, "value": whole_job_mvis(nvis, world, ms), "unit": "Mvis/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32c",
        "data": "synthetic (seeded; 62 stations, 8 km, 8 h; channels uniform in 120-180 MHz, "
                "per-channel flagging U(0, 60%), 4 polarisations of a weakly polarised sky)",
        "config": {"workload": f"channel x pol batch: {C} channels x {pols} pols, one "
                               f"{nx}x{nx} grid of {P} w-planes each, support {S}, "
                               f"{nvis} visibilities ({args.per_channel} per channel before "
                               f"flagging)",
                   "graph": "forward replayed as one CUDA graph", "tuning": best,
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)"},
        "forward_ms": fwd, "adjoint_ms": adj,
        "roofline": {"bound": "hbm", "kernel": "whole step (bin, grid, FFT + w-correction, "
                                                "adjoint, degrid)",
                     "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                     "peak_source": f"{peak_kind} hbm copy bandwidth", "traffic": None,
                     "algorithmic_bytes_per_launch": ab_step},
        "sequential_single_image": {"ms_per_step": seq_ms, "jobs": len(jobs),
                                    "batch_speedup": seq_ms / ms},
        "autotune": {"best": best, "tried": tried},
        "gpu_launches": args.steps * 12,   # 9 forward kernels (graph) + 3 adjoint
        "clocks": clk, "binning": stats, "device_bytes": B.device_bytes(), "gen_s": gen_s,
        "e2e": {"value": nvis / e2e_s / 1e6, "unit": "Mvis/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3, "steps": n_e2e,
                "pipelined": "uploads overlap the previous adjoint, downloads the next kernels",
                "blocking": {"value": nvis / blocking_s / 1e6, "ms_per_step": blocking_s * 1e3}},
        "cells": cells,
    }


# ---------------------------------------------------------------------------
# the large single image, validated on a window and a subset
# ---------------------------------------------------------------------------

def bench_large(args, rank, world, peak, peak_kind):
    """8192^2 x 128 planes (complex64, 69 GB), support 9, 400M visibilities:
    FP32C forward + adjoint timed like the default workload; then a random
    subset's forward image on a window, and the adjoint of an image supported
    on that window, against the FP64 oracle's windowed forms."""
    import torch
    from lofar_gb300 import Plan, synth
    from oracle import oracle as O

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    gen = dict(synth.CONFIGS["c5"]["gen"])
    gen["n_vis"] = args.nvis
    t0 = time.time()
    d = synth.observe_device(device="cuda", **gen)
    gen_s = time.time() - t0
    ins = tuple(d[k] for k in ("uu", "vv", "ww", "vis_real", "vis_img", "weight"))
    n, nx, P, S = d["n"], args.nx, args.planes, args.support
    plan = Plan(nx, nx, P, S, precision="fp32c")
    plan.set_wcorrection(d["resolution"], d["wmin"], d["wmax"])
    plan.set_layout(d["n_baselines"])   # the generator writes [dump][baseline]
    plan.reserve(n)
    image = torch.empty((nx, nx), dtype=torch.complex64, device="cuda")
    out = torch.empty(n, dtype=torch.complex64, device="cuda")
    run_plan_steps(plan, ins, image, out, args.warmup, False)
    stats = plan.stats()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    total_ms, per = run_plan_steps(plan, ins, image, out, args.steps, True)
    clk = clocks.stop()
    ms = max_over_ranks(total_ms, world) / args.steps
    stages = roofline(per, n, nx, P, 8, peak, peak_kind)
    if rank != 0:
        return None
    plan_bytes = plan.device_bytes()
    del out
    torch.cuda.empty_cache()

    # validation on a random subset: FP32C and FP64 on the device over the
    # whole image, and both against the FP64 oracle on a window
    m_sub = min(n, args.subset)
    rng = np.random.default_rng(11)
    sel = torch.as_tensor(np.sort(rng.choice(n, m_sub, replace=False)), device="cuda")
    sub = [x.index_select(0, sel).contiguous() for x in ins]
    host = [x.cpu().numpy() for x in sub]
    wn = min(args.window, nx // 2)
    # finite w-correction (pixel coordinate (iu - N/2) mod N small,
    # phase_correction.cu:164-169) and away from the grid's Nyquist pixel N/2,
    # where the Gaussian kernel's response is ~5e-5
    x0 = y0 = 13 * nx // 16 - wn // 2
    kw = dict(num_w_planes=P, dx=1 / nx, dw=1 / P, w_support=S, nx=nx, ny=nx,
              resolution=d["resolution"], wmin=d["wmin"], wmax=d["wmax"])
    yw = rng.standard_normal((wn, wn)) + 1j * rng.standard_normal((wn, wn))
    imgs, adjs = {}, {}
    _GRIDS.pop(id(plan), None)
    plan.close()
    del plan, image
    for prec in ("fp32c", "fp64"):
        torch.cuda.empty_cache()
        p = Plan(nx, nx, P, S, precision=prec)
        p.set_wcorrection(d["resolution"], d["wmin"], d["wmax"])
        imgs[prec] = p.image_forward(*sub).to(torch.complex64 if prec == "fp32c" else torch.complex128)
        full = torch.zeros((nx, nx), dtype=p.cdtype, device="cuda")
        full[y0:y0 + wn, x0:x0 + wn] = torch.as_tensor(yw, device="cuda").to(p.cdtype)
        adjs[prec] = p.image_adjoint(full).cpu().numpy().astype(np.complex128)
        del full
        p.close()
    a64 = imgs["fp64"]
    a32 = imgs["fp32c"].to(torch.complex128)
    fin = torch.isfinite(a64.real)
    rms = float(torch.sqrt((a64[fin].abs() ** 2).mean()))
    glob = float(torch.sqrt(((a32 - a64)[fin].abs() ** 2).mean())) / rms
    nan_equal = bool(torch.equal(fin, torch.isfinite(a32.real)))
    win32 = a32[y0:y0 + wn, x0:x0 + wn].cpu().numpy()
    win64 = a64[y0:y0 + wn, x0:x0 + wn].cpu().numpy()
    del imgs, a32, a64
    torch.cuda.empty_cache()
    t0 = time.time()
    re, im = O.image_window(*host, x0=x0, y0=y0, wx=wn, wy=wn, **kw)
    t_fwd = time.time() - t0
    ref = re + 1j * im
    t0 = time.time()
    a = O.adjoint_window(yw.real, yw.imag, host[0], host[1], host[2], x0=x0, y0=y0, **kw)
    t_adj = time.time() - t0
    aref = a[:, 0] + 1j * a[:, 1]

    def rel(x, r):
        return float(np.sqrt(np.mean(np.abs(x - r) ** 2) / np.mean(np.abs(r) ** 2)))
    win_err = float(np.sqrt(np.mean(np.abs(win32 - ref) ** 2)))
    validation = {
        "subset": m_sub, "window": [x0, y0, wn, wn],
        "fp32c_vs_fp64_image_rel_rms": glob, "nan_mask_equal": nan_equal,
        "fp64_window_vs_oracle_rel_rms": rel(win64, ref),
        "fp32c_window_vs_oracle_rms_over_image_rms": win_err / rms,
        "fp32c_window_vs_oracle_rel_rms": rel(win32, ref),
        "window_rms_over_image_rms": float(np.sqrt(np.mean(np.abs(ref) ** 2))) / rms,
        "fp64_adjoint_vs_oracle_rel_rms": rel(adjs["fp64"], aref),
        "fp32c_adjoint_vs_oracle_rel_rms": rel(adjs["fp32c"], aref),
        "oracle_seconds": {"forward": t_fwd, "adjoint": t_adj},
        "oracle": "FP64 windowed forms of the oracle (per-plane gridding, row FFT, DFT to the "
                  "window, w-correction; adjoint likewise)",
    }
    g_ = stages["gridding(bin+grid)"]
    return {
        "metric": METRIC, "value": whole_job_mvis(n, world, ms), "unit": "Mvis/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32c",
        "data": "synthetic (seeded; 62 stations, 8 km, 12 h, 20 point sources + noise; "
                "generated on the device)",
        "config": {"workload": f"large single image: {nx}x{nx} grid, {P} w-planes "
                               f"(complex64, {P * nx * nx * 8 / 1e9:.1f} GB), support {S}, "
                               f"{n} visibilities",
                   "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)"},
        "roofline": {"bound": "hbm", "kernel": "gridding stage (bin_count+bin_scan+bin_scatter+grid)",
                     "achieved": g_["gbs"], "peak": peak, "unit": "GB/s", "frac": g_["frac"],
                     "peak_source": f"{peak_kind} hbm copy bandwidth",
                     "traffic": None, "algorithmic_bytes_per_launch": g_["bytes"]},
        "stages": stages,
        "validation": validation,
        "gpu_launches": args.steps * sum(OUR_KERNELS_PER_STEP.values()),
        "clocks": clk, "binning": stats, "plan_device_bytes": plan_bytes,
        "gen_s": gen_s,
    }


def bench_sectoring(vv, ny, support, reps=5):
    """v-slab lists of the reference's multi-rank decomposition (wsg_sector_count
    + wsg_sector_lists) on the device rows, for 16 and 256 slabs: median ms and
    algorithmic GB/s (vv read once, the list entries and offsets written)."""
    import torch
    from lofar_gb300 import sectors
    out = {}
    for S in (16, 256):
        yaxis, dx = ny // S, 1.0 / ny
        wsh = sectors.w_supporth(support, dx)
        times, entries = [], 0
        for _ in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record()
            _, off, index = sectors.sector_lists(vv, S, yaxis, dx, wsh)
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
            entries = int(off[-1])
            del index
        ms = statistics.median(times[1:])
        nbytes = 8 * vv.numel() + 8 * entries + 8 * (S + 2)
        out[f"{S}_slabs"] = {"ms": ms, "entries": entries, "GBps": nbytes / ms / 1e6,
                             "note": "count + lists calls, each with its own scan and host sync"}
    return out


def bench_driver(args, rank, world, peak, peak_kind):
    """The reference's main() on files (wsg_run_paramfile): the c2 observation
    written as a reference dataset directory (meta.txt + six binary files, plus
    the 1000 rows the reader drops), then per step: read, upload, bin, grid,
    per-plane FFT, w-correct, download and write the image dump.  FP64 (the
    reference's arithmetic) and FP32C.  Stage times are the driver's wall
    clock; the files are in the page cache after the first read."""
    import shutil
    import tempfile

    import torch
    from lofar_gb300 import binms, synth
    from oracle import binms_oracle as B

    dev = rank % max(1, torch.cuda.device_count())
    torch.cuda.set_device(dev)
    gen = dict(synth.CONFIGS["c2"]["gen"])
    gen["n_vis"] = args.nvis
    d = synth.observe_device(device="cuda", **gen)
    n, nx, P, S = d["n"], args.nx, args.planes, args.support
    tmp = tempfile.mkdtemp(prefix="wstack_driver_", dir=args.driver_dir)
    try:
        ds = os.path.join(tmp, "ds0") + "/"
        pad = {"uu": 0.5, "vv": 0.5, "ww": 0.5, "weight": 1.0, "vis_real": 0.0, "vis_img": 0.0}
        host = {}
        for k, v in pad.items():
            a = d[k].cpu().numpy()
            host[k] = np.concatenate([a, np.full(1000, v, a.dtype)])
        binms.write_dataset(ds, uu=host["uu"], vv=host["vv"], ww=host["ww"],
                            weights=host["weight"], vis_real=host["vis_real"],
                            vis_img=host["vis_img"], freq_per_chan=1, polarisations=1,
                            baselines=d["n_baselines"], uvmin=d["uvmin"], uvmax=d["uvmax"],
                            wmin=d["wmin"], wmax=d["wmax"])
        bytes_in = sum(os.path.getsize(os.path.join(ds, f)) for f in os.listdir(ds))
        del host
        sectoring = bench_sectoring(d["vv"], args.nx, S)
        del d
        torch.cuda.empty_cache()
        pf = os.path.join(tmp, "paramfile.txt")
        with open(pf, "w") as f:
            f.write(f"ndatasets 1\nDatapath1 {ds}\nnum_threads 1\nw_support {S}\n"
                    f"grid_size_x {nx}\ngrid_size_y {nx}\nnum_w_planes {P}\n"
                    "ufile ucoord.bin\nvfile vcoord.bin\nwfile wcoord.bin\n"
                    "weightsfile weights.bin\nvisrealfile visibilities_real.bin\n"
                    "visimgfile visibilities_img.bin\nmetafile meta.txt\n"
                    "outfile2 grid_real.bin\noutfile3 grid_img.bin\nfftfile2 fft_real.bin\n"
                    "fftfile3 fft_img.bin\ntimingfile timings.dat\n")
        out = os.path.join(tmp, "out")
        os.makedirs(out)
        res = {}
        clocks = ClockSampler(dev)
        clocks.start()
        for prec in ("fp64", "fp32c"):
            for _ in range(args.warmup):
                binms.run(pf, write_image=True, precision=prec, outdir=out)
            reps = [binms.run(pf, write_image=True, precision=prec, outdir=out)
                    for _ in range(args.steps)]
            med = {k: statistics.median(r[k] for r in reps)
                   for k in ("setup", "compose", "kernel", "fft", "phase", "write", "total")}
            res[prec] = {"mvis_s": n / med["total"] / 1e6, "stages_s": med,
                         "read_GBps": bytes_in / med["setup"] / 1e9,
                         "dropped": reps[-1]["dropped"]}
        clk = clocks.stop()
        if args.driver_write_data:
            r = binms.run(pf, write_data=True, precision="fp32c", outdir=out)
            cube = 2 * 2 * P * nx * nx * 8   # two dumps, two float64 files each
            res["write_data_fp32c"] = {"write_s": r["write"], "dump_bytes": cube,
                                       "dump_GBps": cube / r["write"] / 1e9,
                                       "total_s": r["total"]}
        # the oracle port of the reader on the same files (one thread)
        t = time.perf_counter()
        prm = B.parse_parameter_file(open(pf).read())
        meta, start = B.partition(B.parse_metadata(open(ds + "meta.txt").read()))
        B.read_measurements(ds, prm, meta, start)
        cpu_read_s = time.perf_counter() - t
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    ms = max_over_ranks(res["fp64"]["stages_s"]["total"] * 1e3, world)
    if rank != 0:
        return None
    return {
        "metric": "Mvis/s files-to-image through the reference's main() (read + grid + FFT + "
                  "w-correct + image dump)",
        "value": whole_job_mvis(n, world, ms), "unit": "Mvis/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the c2 observation written as a reference dataset directory)",
        "config": {"workload": f"wsg_run_paramfile: {nx}x{nx} grid, {P} w-planes, support {S}, "
                               f"{n} measurements (+1000 dropped) from {bytes_in} bytes of files",
                   "files": "page cache after the first read", "parallelism": f"replicas{world}"},
        "precisions": res, "clocks": clk, "sectoring": sectoring,
        "cpu_baseline": {"value": cpu_read_s, "unit": "s to read the dataset", "cores": 1,
                         "kind": "port", "sample": "the whole dataset through the NumPy reader "
                                                   "restatement (oracle/binms_oracle.py)"},
        "gpu_launches": None,
    }


NOMINAL_FP64_TFLOPS = 1.25   # GB300 dense FP64, nominal (no measured FP64 peak is recorded)


def fft_fp64_equivalent(nx, planes, ms):
    """FP64-equivalent rate of one direction's per-plane 2D FFTs, 5 N log2 N
    flops per N-point plane, over `ms` (the FFT + w-correction stage: a lower
    bound for the FFT alone)."""
    npix = nx * nx
    flop = 5.0 * npix * math.log2(npix) * planes
    tf = flop / (ms * 1e-3) / 1e12
    return {"tflops": tf, "of_nominal_fp64": tf / NOMINAL_FP64_TFLOPS,
            "note": "5 N log2 N per plane over the FFT + w-correction stage time; the FFT "
                    "runs in 64-bit fixed point on the integer pipe; nominal FP64 peak "
                    f"{NOMINAL_FP64_TFLOPS} TFLOP/s"}


def roofline(per, n, nx, P, sc, peak, peak_kind):
    ab = algorithmic_bytes(n, nx, nx, P, sc)
    med = {s: statistics.median(v) for s, v in per.items() if v}
    stages = {}
    grid_ms = med["bin"] + med["grid"]
    stages["gridding(bin+grid)"] = dict(ms=grid_ms, bytes=ab["grid"],
                                        gbs=ab["grid"] / (grid_ms * 1e-3) / 1e9)
    for s in ("fft_wcorrect", "wcorrect_adj_fft", "degrid"):
        stages[s] = dict(ms=med[s], bytes=ab[s], gbs=ab[s] / (med[s] * 1e-3) / 1e9)
    for v in stages.values():
        v["frac"] = v["gbs"] / peak
    stages["bin"] = dict(ms=med["bin"])
    stages["grid_kernel"] = dict(ms=med["grid"])
    return stages


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "ours":
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
            dist.init_process_group("nccl")
    if args.impl == "reference":
        line = bench_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line))
        return 0

    import torch
    peak, peak_kind = peaks()
    if args.workload in ("c4", "c5", "driver"):
        fn = {"c4": bench_batch, "c5": bench_large, "driver": bench_driver}[args.workload]
        line = fn(args, rank, world, peak, peak_kind)
        if line is not None:
            print(json.dumps(line))
        return 0
    res, obs = bench_ours(args, rank, world)
    if rank != 0:
        return 0
    sc = 8
    n = res["n"]
    stages = roofline(res["per"], n, args.nx, args.planes, sc, peak, peak_kind)
    g = stages["gridding(bin+grid)"]
    line = {
        "metric": METRIC,
        "value": res["value"],
        "unit": "Mvis/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": res["ms_per_step"],
        "higher_is_better": True,
        "scaling": "strong" if "planes" in res else "weak",
        "vs_baseline": None,
        "dtype": "fp32c",
        "data": (f"synthetic (seeded; {obs.meta['n_stations']} stations in a "
                 f"{obs.meta['diameter_m'] / 1000:g} km disk, {obs.meta['hours']:g} h earth-rotation "
                 "tracks, 20 point sources + noise)"),
        "config": {"workload": f"w-stacking fwd+adjoint, {args.nx}x{args.nx} grid, {args.planes} "
                               f"w-planes, support {args.support}, {n} visibilities "
                               + ("in one image over all GPUs" if "planes" in res else "per GPU"),
                   "precision": "FP32 complex grid, int32 fixed-point tile sums, FP64-exact "
                                "coordinates and phase argument",
                   "parallelism": (f"planes{world}" if "planes" in res else f"replicas{world}"),
                   "l2": res.get("l2", "inputs larger than L2 (no flush)"),
                   "binning": res.get("layout", "index order")},
        "roofline": {"bound": "hbm", "kernel": "gridding stage (bin_count+bin_scan+bin_scatter+grid)",
                     "achieved": g["gbs"], "peak": peak, "unit": "GB/s", "frac": g["frac"],
                     "peak_source": f"{peak_kind} hbm copy bandwidth",
                     "traffic": profiled_traffic(res["stats"]["records"]),
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                       "stage's kernels (profiles/launches_fwd_adj_4096x32_50M.md),"
                                       " scaled by records",
                     "algorithmic_bytes_per_launch": g["bytes"]},
        "stages": stages,
        "gpu_launches": args.steps * sum(OUR_KERNELS_PER_STEP.values()),
        "clocks": res["clocks"],
        "binning": res["stats"],
        "plan_device_bytes": res["plan_bytes"],
    }
    if "fp64" in res:
        f = res["fp64"]
        line["fp64"] = {"value": f["value"], "unit": "Mvis/s", "ms_per_step": f["ms_per_step"],
                        "steps": args.fp64_steps,
                        "fp32c_over_fp64": res["value"] / f["value"],
                        "image_rel_rms_err": f["image_rel_rms"],
                        "image_rel_max_err": f["image_rel_max"],
                        "nan_mask_equal": f["nan_mask_equal"],
                        "grid_plane_rel_rms_err_max": f["plane_rel_rms_max"],
                        "stages_ms": {s: statistics.median(v) for s, v in f["per"].items() if v},
                        # complex128 cube; the FP64 form runs its taps, FFT and
                        # w-correction in 64-bit fixed point, so its stages are
                        # bound by integer (and FP64 exponential) issue, not HBM
                        "stages": roofline(f["per"], n, args.nx, args.planes, 16, peak, peak_kind),
                        "fft_fp64_equivalent": fft_fp64_equivalent(
                            args.nx, args.planes,
                            statistics.median(f["per"]["fft_wcorrect"]))}
    if "e2e" in res:
        line["e2e"] = res["e2e"]
    if "planes" in res:
        line["e2e"] = {"value": None, "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0,
                       "note": "not measured in the plane-sharded form (run N=1 for e2e)"}
    if not args.no_cpu and world >= 1:
        line["cpu_baseline"] = cpu_baseline(obs, res["res"], args,
                                            steps=3 if args.workload == "c1" else 1)
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
