"""Benchmark of the SRRF radiality path on one GB300 (or N replicas).

Workload (default, "mid"): 100 volumes of 128x128x64 uint16 (filament-like
synthetic scene, seed 1235), magnification 4x4x2 (512x512x128 output), ring
radius 0.5, 12 ring axes (AxesinRing 6), smoothed gradient with ranges 1,
TRAC-2 (ITC 0) with intensity weighting. One step = one full forward over the
whole series: fused gradient+interpolation+radiality kernel, then the temporal
reduction.

Printed JSON line (rank 0):
  value    output voxel-volumes per second, inputs already in HBM, device time
           (CUDA events on the launching stream) over exactly --steps steps;
  e2e      the same metric through the C-ABI entry point with pinned host
           buffers (host->device input copy and device->host map copy inside
           the timed region);
  roofline FP32 throughput of the radiality kernel: algorithmic flops of the
           separable method per launch / average launch time, against the
           nominal FP32 FMA peak at the measured maximum SM clock;
  cpu_baseline  the FP32 CPU port of the reference radiality loop (oracle/,
           OpenMP over all host cores) timed on a bounded sub-slab.
  reference_gpu  the reference's own CUDA kernels (kernel.cu built for sm_103a
           into baseline/_ref, driven as its host code drives them) on this
           GPU, on the small and the 216-block batching series, next to this
           library (the reference has one magnification for all axes and int
           index arithmetic, so it cannot run the mid workload itself).
--impl reference times the CPU port alone, on the mid workload.
"""
from __future__ import annotations

import argparse
import ctypes
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

WORKLOAD = dict(name="mid", T=100, shape=(128, 128, 64), mag=(4, 4, 2), method=3, itc=0, trac_order=2)
CFG_KW = dict(mag=(4, 4, 2), method=3, itc=0, trac_order=2, gradient_smooth=1, main_range=1, x_range=1,
              y_range=1, z_range=1, intensity_w=1, axes_in_ring=6, ring_radius=0.5)
# CPU sample: a fine sub-slab of the same workload, all time points
CPU_REGION_LO = (240, 240, 56)
CPU_REGION_HI = (272, 272, 72)
# per-step sample of the reference arm (smaller, so K + W steps stay short)
REF_REGION_LO = (240, 240, 56)
REF_REGION_HI = (256, 256, 64)


def max_over_ranks(x: float) -> float:
    """Maximum of a per-rank time over all ranks (identity without a process
    group); the tensor lives where the backend wants it (CUDA for NCCL)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world_size: int, seconds_max: float) -> float:
    """Replicas (weak scaling): every rank runs the whole workload; the job rate is
    all ranks' units over the slowest rank's time."""
    return units_per_rank * world_size / seconds_max


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_input(volumes=None):
    from rfba_gb300 import synth
    x, _ = synth.workload("mid", n_vol=volumes)
    return x


def algorithmic_flops_per_voxel_volume(cfg) -> dict:
    """Flops per output voxel-volume of the separable method as implemented
    (rfba_gb300.srrf.flops_per_voxel_volume), with the direct forms for
    reference: the reference executes ~90,700 per voxel-volume (144 samples x 3
    x 64-tap interpolations with recomputed weights); over the 62 distinct points
    the direct form is ~39,300."""
    from rfba_gb300 import srrf
    info = srrf.plan_info(cfg)
    return {"separable": srrf.flops_per_voxel_volume(cfg), **info,
            "direct_distinct": 39300.0, "direct_reference": 90700.0}


def fp32_peak_tflops(sm_count: int, sm_mhz: float) -> float:
    return sm_count * 128 * 2 * sm_mhz * 1e6 / 1e12


def cpu_baseline(x: np.ndarray, reps: int = 1):
    """FP32 CPU port of the reference radiality loop on a sub-slab (all T)."""
    from oracle import oracle as O
    oc = O.make_conf(**{k: v for k, v in CFG_KW.items()})
    xf = x.astype(np.float32)
    lo, hi = CPU_REGION_LO, CPU_REGION_HI
    n_vox = int(np.prod(np.array(hi) - np.array(lo)))
    t0 = time.perf_counter()
    for _ in range(reps):
        O.srrf_region(xf, oc, lo, hi, dtype=np.float32)
    dt = time.perf_counter() - t0
    units = n_vox * x.shape[0] * reps
    return {"value": units / dt, "unit": "voxel-volumes/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"fine region x{lo[0]}:{hi[0]} y{lo[1]}:{hi[1]} z{lo[2]}:{hi[2]} of the 512x512x128 map, "
                      f"all {x.shape[0]} volumes ({units} voxel-volumes, {dt:.1f} s); FP32 port of kernel.cu "
                      f"(all 144 ring samples, OpenMP over subvoxels)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    x = make_input()
    oc = O.make_conf(**CFG_KW)
    xf = x.astype(np.float32)
    lo, hi = REF_REGION_LO, REF_REGION_HI
    n_vox = int(np.prod(np.array(hi) - np.array(lo)))
    for _ in range(args.warmup):
        O.srrf_region(xf, oc, lo, hi, dtype=np.float32)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.srrf_region(xf, oc, lo, hi, dtype=np.float32)
    dt = time.perf_counter() - t0
    units = n_vox * x.shape[0] * args.steps
    v = units / dt
    line = {
        "impl": "reference", "metric": "radiality voxel-volumes/s", "value": v, "unit": "voxel-volumes/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "mid: 100 x 128x128x64 u16, mag 4x4x2, TRAC-2 ITC0, 12 axes, r 0.5",
                   "sample": f"fine region {lo}-{hi}, all volumes"},
        "cpu_baseline": {"value": v, "unit": "voxel-volumes/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"fine region {lo}-{hi} of the 512x512x128 map, all 100 volumes per step; "
                                   "FP32 port of the reference kernel.cu radiality loop, OpenMP over all cores"},
        "e2e": {"value": v, "unit": "voxel-volumes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _batching_case(ctx, x, cfg, steps: int, label: str) -> dict:
    """One batching measurement: doSplit's 29-voxel blocks with a 1-voxel
    overlap over the whole series; the batched path (one persistent launch per
    pass, autotuned schedule, replayed as a CUDA graph) on device buffers and
    through the C-ABI with pinned host buffers, against the plain path (one
    launch sequence per block with that block's host<->device copies)."""
    import torch
    from rfba_gb300 import srrf
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 29, 1)
    units = oe * x.shape[0]
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    outd = torch.empty(oe, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    t0 = time.perf_counter()
    ctx.forward_blocks(cfg, xd, blocks, n, oe, out=outd, stream=stream.cuda_stream)  # autotune + capture
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    sched = ctx.schedule()
    ctx.forward_blocks(cfg, xd, blocks, n, oe, out=outd, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.forward_blocks(cfg, xd, blocks, n, oe, out=outd, stream=stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    replay = ctx.schedule()
    dev_ms = e0.elapsed_time(e1) / steps
    pin_in = torch.empty(x.nbytes, dtype=torch.uint8).pin_memory().numpy().view(np.uint16).reshape(x.shape)
    pin_in[...] = x
    pin_out = torch.empty(oe, dtype=torch.float32).pin_memory().numpy()
    ctx.forward_blocks(cfg, pin_in, blocks, n, oe, out=pin_out)
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.forward_blocks(cfg, pin_in, blocks, n, oe, out=pin_out)
    e2e_ms = (time.perf_counter() - t0) / steps * 1e3
    plain_out = np.zeros(oe, np.float32)
    ctx.forward_blocks_plain(cfg, x, blocks, n, oe, out=plain_out)  # warm
    t0 = time.perf_counter()
    ctx.forward_blocks_plain(cfg, x, blocks, n, oe, out=plain_out)
    plain_ms = (time.perf_counter() - t0) * 1e3
    same = bool(np.array_equal(np.nan_to_num(plain_out), np.nan_to_num(pin_out)) and
                np.array_equal(np.isnan(plain_out), np.isnan(pin_out)))
    edges = sorted({int(blocks[i].size[a]) for i in range(n) for a in range(3)})
    return {"case": label, "blocks": n, "block_edges": edges, "voxel_volumes": units,
            "schedule": {"tile_rows": sched["tile_rows"], "tile_order": sched["tile_order"],
                         "graph_replay": replay["graph"], "first_call_s": first_s},
            "batched_device_ms": dev_ms, "batched_e2e_ms": e2e_ms, "plain_per_block_ms": plain_ms,
            "batched_device_value": units / (dev_ms / 1e3), "batched_e2e_value": units / (e2e_ms / 1e3),
            "plain_value": units / (plain_ms / 1e3), "speedup_device_vs_plain": plain_ms / dev_ms,
            "speedup_e2e_vs_plain": plain_ms / e2e_ms, "batched_equals_plain": same}


def measure_batching(ctx, steps: int) -> dict:
    """Batching workload: 50 volumes (3000 filament emitters) at magnification
    3, cut by doSplit's rule (29, 1-voxel overlap). 160x160x160 gives the 216
    blocks (edges 25 and 29) of the batching config, measured with the temporal
    mean and with TRAC-2; the literal 160x160x120 series gives 180 blocks."""
    from rfba_gb300 import srrf, synth
    kw = dict(mag=3, gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)
    x, _ = synth.workload("batching", shape=(160, 160, 160))
    cases = [_batching_case(ctx, x, srrf.Config.make(method=1, **kw), steps, "160^3 TRA"),
             _batching_case(ctx, x, srrf.Config.make(method=3, itc=0, trac_order=2, **kw), steps, "160^3 TRAC-2")]
    x, _ = synth.workload("batching")
    cases.append(_batching_case(ctx, x, srrf.Config.make(method=1, **kw), steps, "160x160x120 TRA"))
    head = cases[0]
    return {"workload": "batching: 50 volumes, 3000 filament emitters, doSplit 29/1 blocks, mag 3", **head,
            "cases": cases}


def measure_reference_gpu(ctx, sample_blocks: int = 8) -> dict:
    """The reference's own CUDA kernels (kernel.cu, compiled for sm_103a) on this
    GPU, driven as SRRFGradientCalcGPU and the GradientCalc.cpp block loop drive
    them (baseline/refgpu.py), next to this library on the same inputs:
    (1) the small series (30 x 32^3 u16, mag 2, temporal mean with intensity
    weighting) as one call; (2) the 216-block batching series (50 x 160^3, mag 3,
    doSplit 29/1 blocks, temporal mean), the reference's per-block loop timed on
    the first `sample_blocks` blocks (all 50 volumes) and scaled to all blocks by
    voxel-volumes. Each part reports the relative L-inf difference of the maps."""
    import torch
    from baseline import refgpu
    from rfba_gb300 import srrf, synth
    from tests.parity import rel_linf
    if not refgpu.available():
        return {"unavailable": "baseline/_ref cubin not built (needs the reference sources where build() runs)"}
    ref = refgpu.RefGPU(0)
    res = {}
    try:
        kw = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1, method=1, intensity_w=1)
        cfg = srrf.Config.make(mag=2, **kw)
        x, _ = synth.workload("small")
        xf = x.astype(np.float32)
        ref.gradient_calc_gpu(xf, cfg)
        rmap, st = ref.gradient_calc_gpu(xf, cfg)
        xd = torch.from_numpy(x.view(np.int16)).cuda()
        out = ctx.forward(cfg, xd)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            ctx.forward(cfg, xd, out=out)
        e1.record()
        torch.cuda.synchronize()
        ours_ms = e0.elapsed_time(e1) / 5
        units = int(np.prod(rmap.shape)) * x.shape[0]
        res["small"] = {"workload": "30 x 32^3 u16 -> 64^3 map, mag 2, TRA (IW), one call",
                        "reference_kernel_ms": st["kernel_ms"], "reference_call_ms": st["call_ms"],
                        "ours_device_ms": ours_ms,
                        "reference_kernel_value": units / (st["kernel_ms"] / 1e3),
                        "ours_device_value": units / (ours_ms / 1e3),
                        "speedup_kernels": st["kernel_ms"] / ours_ms,
                        "nan_masks_equal": bool(np.array_equal(np.isnan(rmap), np.isnan(out.cpu().numpy()))),
                        "rel_linf_vs_reference": rel_linf(out.cpu().numpy(), rmap)}

        cfg = srrf.Config.make(mag=3, **kw)
        x, _ = synth.workload("batching", shape=(160, 160, 160))
        blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 29, 1)
        ours = ctx.forward_blocks(cfg, x, blocks, n, oe)
        k = min(sample_blocks, n)
        rout = np.full(oe, np.nan, np.float32)
        ref.gc_block_loop(x, cfg, blocks, 1, rout)  # warm
        st = ref.gc_block_loop(x, cfg, blocks, k, rout)
        mask = np.zeros(oe, bool)
        for i in range(k):
            b = blocks[i]
            mask[b.out_offset:b.out_offset + int(np.prod([b.hi[a] - b.lo[a] for a in range(3)]))] = True
        units_sample = int(mask.sum()) * x.shape[0]
        units_all = oe * x.shape[0]
        scale = units_all / units_sample
        res["batching_216"] = {
            "workload": "50 x 160^3 u16, doSplit 29/1 blocks (216), mag 3, TRA (IW)",
            "sample": f"reference per-block loop on blocks 0-{k - 1} of {n}, all 50 volumes, "
                      f"scaled by voxel-volumes x{scale:.1f}",
            "reference_plain_wall_ms_est": st["wall_ms"] * scale,
            "reference_plain_kernel_ms_est": st["kernel_ms"] * scale,
            "reference_plain_value": units_sample / (st["wall_ms"] / 1e3),
            "reference_kernel_value": units_sample / (st["kernel_ms"] / 1e3),
            "nan_masks_equal": bool(np.array_equal(np.isnan(rout[mask]), np.isnan(ours[mask]))),
            "rel_linf_vs_reference": rel_linf(ours[mask], rout[mask])}
    finally:
        ref.close()
    return res


def measure_threeb(ctx, steps: int = 20) -> dict:
    """3B spot gradient (SpotNegProbabilityDiffWithSampledBackground,
    multispot5.cc:616-664) on one 29^3 block: 10 background samples (the
    shipped main.gibbs.samples), 100 frames, 24,389 mask voxels, the shipped
    3-state model; FP64. Device: data resident, the spot moved every call (the
    conjugate-gradient optimiser's pattern); e2e: samples and data copied from
    host memory every call; CPU: the FP64 oracle (the reference's operation
    order, samples over threads like the reference) on all host cores."""
    import torch
    from rfba_gb300 import srrf, synth
    S, F, shape = 10, 100, (29, 29, 29)
    bg, pix, px, spot = synth.threeb_block(77, S, F, shape)
    model = srrf.ThreeBModel.make([[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]], [0.5, 0.5, 0.0],
                                  variance=1.0, z_factor=1.0)
    d = [torch.from_numpy(a).cuda() for a in (bg, pix, px)]
    g, _ = ctx.spot_gradient_3b(model, *d, spot)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(steps):
        g, _ = ctx.spot_gradient_3b(model, *d, spot + 1e-3 * k)
    dev_ms = (time.perf_counter() - t0) / steps * 1e3
    pin = [torch.from_numpy(a).pin_memory().numpy() for a in (bg, pix, px)]
    ctx.spot_gradient_3b(model, *pin, spot)
    t0 = time.perf_counter()
    for k in range(steps):
        g_h, _ = ctx.spot_gradient_3b(model, *pin, spot + 1e-3 * k)
    e2e_ms = (time.perf_counter() - t0) / steps * 1e3
    res = {"workload": "3B spot gradient: 10 samples x 100 frames x 29^3 mask voxels, FP64",
           "device_ms": dev_ms, "device_value": 1e3 / dev_ms, "e2e_ms": e2e_ms, "e2e_value": 1e3 / e2e_ms,
           "unit": "spot-gradient evaluations/s", "h2d_bytes_per_call": int(bg.nbytes + pix.nbytes + px.nbytes),
           "fp64_flops_per_call": int(S * F * np.prod(shape) * 18)}
    res["fp64_tflops_device"] = res["fp64_flops_per_call"] / (dev_ms * 1e-3) / 1e12
    # one spot optimisation as 3B runs it (multispot5.cc:1614-1636): the shipped
    # main.cg.max_iterations 5 and cg.max_motion 0.5 with the brightness limit
    # scaled by the prior's std; samples and data copied in once per spot
    lim = threeb_motion_limit()
    ctx.optimise_spot_3b(model, *pin, spot, lim, 5)
    t0 = time.perf_counter()
    x_opt, it, ev = ctx.optimise_spot_3b(model, *pin, spot, lim, 5)
    opt_ms = (time.perf_counter() - t0) * 1e3
    res["optimise"] = {"what": "one spot optimisation (ConjugateGradientOnly<5>, 5 line searches, max motion 0.5), "
                               "samples and data copied from pinned host memory once",
                       "ms": opt_ms, "line_searches": it, "gradient_evaluations": ev,
                       "ms_per_evaluation": opt_ms / max(ev, 1), "spot": x_opt.tolist()}
    res.update(measure_gibbs(ctx))
    return res


THREEB_BLOCK = dict(seed=91, F=100, shape=(29, 29, 29), K=20)


def _gibbs_block():
    """The 3B block of the sampler / fit timings: 20 blinking spots in a 29^3
    block over 100 frames, normalised as 3B's preprocessing leaves data (no
    background, unit noise)."""
    from rfba_gb300 import synth
    b = THREEB_BLOCK
    return synth.threeb_spots_block(b["seed"], b["F"], b["shape"], b["K"], background=0.0)


def _threeb_model():
    from rfba_gb300 import srrf
    return srrf.ThreeBModel.make([[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]], [0.5, 0.5, 0.0],
                                 variance=1.0, z_factor=1.0, mu_brightness=3.5, sigma_brightness=1.0,
                                 mu_blur=0.12869, sigma_blur=0.1)


def measure_gibbs(ctx) -> dict:
    """3B's Gibbs sampler, free energy, one main-loop pass, the sampled-background
    Hessian and one model modification on a 29^3 block with 20 spots and 100
    frames (multispot5.cfg's settings: gibbs.mixing_iterations 1,
    main.gibbs.samples 10, add_remove.thermo.samples 1000,
    main.cg.max_iterations 5, cg.max_motion 0.5, position.extra_radius 2.3,
    add_remove.hessian.outer / inner samples 100 / 1000): GPU wall time per
    call, data from host memory (the Hessian's 100 draws already on the
    device)."""
    from rfba_gb300 import srrf
    pix, pixels, spots = _gibbs_block()
    m = _threeb_model()
    K, F = len(spots), pix.shape[0]
    masks = srrf.spot_masks_3b(pixels, spots)
    ctx.gibbs_sample_3b(m, pix, pixels, spots, masks, n_draws=10, seed=1)
    t0 = time.perf_counter()
    reps = 5
    for r in range(reps):
        ctx.gibbs_sample_3b(m, pix, pixels, spots, masks, n_draws=10, seed=2 + r)
    g_ms = (time.perf_counter() - t0) / reps * 1e3
    t0 = time.perf_counter()
    fe, _ = ctx.free_energy_3b(m, pix, pixels, spots, masks, samples=1000, seed=3)
    fe_ms = (time.perf_counter() - t0) * 1e3
    lim = threeb_motion_limit(3.5, 1.0, 0.5)
    ctx.optimise_pass_3b(m, pix, pixels, spots[:2], 0, 10, 1, 5, lim, 2.3, seed=4)  # warm-up
    t0 = time.perf_counter()
    out, ev = ctx.optimise_pass_3b(m, pix, pixels, spots, 0, 10, 1, 5, lim, 2.3, seed=5)
    pass_ms = (time.perf_counter() - t0) * 1e3
    # the sampled-background Hessian at spot 0 on 100 draws (add_remove.hessian
    # outer / inner samples 100 / 1000), the draws' intensities staged on the device
    import torch
    _, bg = ctx.gibbs_sample_3b(m, pix, pixels, spots, masks, n_draws=100, seed=6, exclude_spot=0,
                                want_states=False)
    bg_d, pix_d, px_d = (torch.from_numpy(a).cuda() for a in (bg, pix, pixels))
    del bg
    ctx.spot_hessian_3b(m, bg_d, pix_d, px_d, spots[0], bs_iterations=1000, seed=7)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in range(3):
        ctx.spot_hessian_3b(m, bg_d, pix_d, px_d, spots[0], bs_iterations=1000, seed=8 + r)
    hess_ms = (time.perf_counter() - t0) / 3 * 1e3
    del bg_d, pix_d, px_d
    torch.cuda.empty_cache()
    # one try of try_modifying_model with the shipped settings
    prm = srrf.ThreeBFitParams.make(lim)
    t0 = time.perf_counter()
    kept, rec = ctx.modify_model_3b(m, pix, pixels, spots, prm, seed=9)
    mod_ms = (time.perf_counter() - t0) * 1e3
    return {"hessian": {"what": f"sampled_background_spot_hessian_ffbs: 100 background draws x 1000 backward "
                                f"samples, {F} frames, {len(pixels)} pixels", "ms": hess_ms},
            "modify": {"what": f"one try of try_modifying_model on {K} spots with multispot5.cfg's settings "
                               "(optimiser 20 draws x 10 attempts with 1000-sample Hessians, Hessian 100 x 1000, "
                               "two free energies of 1000 draws)", "ms": mod_ms, "proposal": "add" if rec["added"]
                       else "remove", "kept_model": rec["kept"], "gradient_evaluations": rec["evaluations"],
                       "spots_after": len(kept)},
            "gibbs": {"what": f"GibbsSampler2 from all spots off: 10 draws x 1 sweep over {K} spots, {F} frames, "
                              f"{len(pixels)} mask voxels (masks {int(masks[0][-1])} voxels in all)",
                      "ms": g_ms, "spot_updates_per_s": 10 * K / (g_ms * 1e-3)},
            "free_energy": {"what": f"NegativeFreeEnergy::compute_with_mask, 1000 thermodynamic samples, {K} spots",
                            "ms": fe_ms, "value": fe},
            "pass": {"what": f"one pass of optimize_each_spot_in_turn over {K} spots (10 Gibbs draws + "
                             "conjugate gradient per spot)", "ms": pass_ms, "gradient_evaluations": ev,
                     "spots_kept": len(out)}}


def threeb_motion_limit(mu: float = 3.5, sigma: float = 1.0, max_motion: float = 0.5):
    """3B's per-parameter step limits (multispot5.cc:1484, storm.h:386-389)."""
    return max_motion * np.array([np.sqrt((np.exp(sigma ** 2) - 1) * np.exp(2 * mu + sigma ** 2)), 1, 1, 1, 1])


def threeb_cpu_baseline(res: dict, reps: int = 3) -> dict:
    """The FP64 oracle of the 3B spot gradient on all host cores (test
    infrastructure, the CPU-baseline leg), on the same block."""
    from oracle import threeb as T
    from rfba_gb300 import synth
    bg, pix, px, spot = synth.threeb_block(77, 10, 100, (29, 29, 29))
    want = T.spot_neg_prob_diff(bg, pix, px, spot, nthreads=os.cpu_count() or 1)
    t0 = time.perf_counter()
    for _ in range(reps):
        T.spot_neg_prob_diff(bg, pix, px, spot, nthreads=os.cpu_count() or 1)
    cpu_ms = (time.perf_counter() - t0) / reps * 1e3
    out = {"cpu_ms": cpu_ms, "cpu_value": 1e3 / cpu_ms, "cores": os.cpu_count(),
           "kind": "port (FP64 oracle, pinned bit for bit to the reference's headers; threads over samples)",
           "speedup_device_vs_cpu": cpu_ms / res["device_ms"], "speedup_e2e_vs_cpu": cpu_ms / res["e2e_ms"],
           "oracle_gradient": want.tolist()}
    if "optimise" in res:
        # the same optimisation with the oracle's gradient on the host cores
        from rfba_gb300 import srrf
        nt = os.cpu_count() or 1
        t0 = time.perf_counter()
        x_cpu, it, ev = srrf.cg_only_run(lambda x: T.spot_neg_prob_diff(bg, pix, px, x, nthreads=nt), spot,
                                         threeb_motion_limit(), 5)
        opt_ms = (time.perf_counter() - t0) * 1e3
        out["optimise"] = {"ms": opt_ms, "gradient_evaluations": ev,
                           "speedup_e2e_vs_cpu": opt_ms / res["optimise"]["ms"],
                           "max_abs_spot_difference": float(np.max(np.abs(x_cpu - np.array(res["optimise"]["spot"]))))}
    if "gibbs" in res:
        out.update(gibbs_cpu_baseline(res))
    return out


def _port_hessian_draws(pix, pixels, spots, moff, midx, si, A, pi):
    """Four GibbsSampler2 draws of the block with spot 0 taken off (the port)."""
    from oracle import gibbs_oracle as G
    st, ints = G.port_run(pix, si, moff, midx, A, pi, 1.0, 1, 4, 11, want_int=True)
    for d in range(4):
        ints[d][st[d, 0] == 0] -= si[0]
    return st, ints


def gibbs_cpu_baseline(res: dict) -> dict:
    """The C++ port of the sampler and of the pass (oracle/gibbs_port.cpp, the
    reference's MT19937 stream and order; the sampler single-threaded as the
    reference's GibbsSampler2::next is, the spot gradient over all host cores)
    on bounded samples of the same workloads, scaled up: the free energy on 20
    of its 1000 draws, the pass on 2 of its 20 spots."""
    from oracle import gibbs_oracle as G
    from rfba_gb300 import srrf
    pix, pixels, spots = _gibbs_block()
    K = len(spots)
    moff, midx = srrf.spot_masks_3b(pixels, spots)
    si = G.spot_intensity(pixels, spots, 1.0)
    A = np.array([[0.16, 0.84, 0.0], [0.495, 0.495, 0.01], [0.0, 0.0, 1.0]])
    pi = np.array([0.5, 0.5, 0.0])
    t0 = time.perf_counter()
    G.port_run(pix, si, moff, midx, A, pi, 1.0, 1, 10, 1)
    g_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    G.port_run(pix, si, moff, midx, A, pi, 1.0, 1, 20, 3)
    fe_ms = (time.perf_counter() - t0) * 1e3 * 1000 / 20
    lim = threeb_motion_limit(3.5, 1.0, 0.5)
    nt = os.cpu_count() or 1
    _, (tg, tc) = G.port_pass(pix, pixels, spots, 0, 10, 1, 5, lim, 2.3, A, pi, 1.0, 1.0, 3.5, 1.0, 0.12869, 0.1, 5,
                              nthreads=nt, max_spots=2)
    pass_ms = (tg + tc) * 1e3 * K / 2
    # the Hessian on 4 of its 100 background draws, scaled by 25
    _, bg4 = _port_hessian_draws(pix, pixels, spots, moff, midx, si, A, pi)
    t0 = time.perf_counter()
    G.port_spot_hessian(bg4, pix, pixels, spots[0], A, pi, 1.0, 1.0, 3.5, 1.0, 0.12869, 0.1, 1000, 8, nthreads=4)
    hess_ms = (time.perf_counter() - t0) * 1e3 * 25
    return {"hessian": {"cpu_ms": hess_ms, "speedup_vs_cpu": hess_ms / res["hessian"]["ms"], "cores": 4,
                        "sample": "4 of 100 background draws on 4 threads (the reference's threads each take draws), "
                                  "scaled by 25", "kind": "port"},
            "gibbs": {"cpu_ms": g_ms, "speedup_vs_cpu": g_ms / res["gibbs"]["ms"], "cores": 1,
                      "kind": "port (draws bit-identical to the reference's GibbsSampler2)"},
            "free_energy": {"cpu_ms": fe_ms, "speedup_vs_cpu": fe_ms / res["free_energy"]["ms"], "cores": 1,
                            "sample": "20 of 1000 draws, scaled by 50"},
            "pass": {"cpu_ms": pass_ms, "speedup_vs_cpu": pass_ms / res["pass"]["ms"], "cores": nt,
                     "sample": "2 of 20 spots, scaled by 10", "cpu_gibbs_s_per_spot": tg / 2,
                     "cpu_optimiser_s_per_spot": tc / 2}}


def measure_diff(ctx, steps: int, iters: int = 20, volumes=None) -> dict:
    """Differentiation workload: 60 volumes of 64^3 float32 (300 emitters) with a
    random-walk drift (sigma 0.15 voxel per step) applied by Catmull-Rom
    resampling; forward = drift correction + SRRF at magnification 2, TRAC-2
    (ITC 0); objective L = -||map||_2. Times forward and forward+adjoint with CUDA
    events, then runs gradient descent on L over the 60 x 3 shifts."""
    import torch
    from rfba_gb300 import drift, srrf, synth
    x, scene = synth.workload("diff", n_vol=volumes)
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=2, gradient_smooth=1, main_range=1, x_range=1,
                           y_range=1, z_range=1)
    T = x.shape[0]
    xd = torch.from_numpy(x).cuda()
    sh = torch.zeros((T, 3), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    units = x.shape[1] * x.shape[2] * x.shape[3] * 8 * T

    objective, grad_map = drift.objective, drift.grad_map

    m = ctx.forward_shifted(cfg, xd, sh, stream=stream.cuda_stream)
    g = grad_map(m)
    ctx.backward(cfg, xd, sh, g, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    for _ in range(steps):
        m = ctx.forward_shifted(cfg, xd, sh, out=m, stream=stream.cuda_stream)
    e1.record(stream)
    for _ in range(steps):
        m = ctx.forward_shifted(cfg, xd, sh, out=m, stream=stream.cuda_stream)
        g = grad_map(m)
        ctx.backward(cfg, xd, sh, g, stream=stream.cuda_stream)
    e2.record(stream)
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / steps
    fwdadj_ms = e1.elapsed_time(e2) / steps
    # Drift refinement: minimise L (maximise the map's norm) over the shifts
    # with Adam. All volumes start from a common half-voxel shift so that every
    # volume is resampled (a volume left on the integer grid escapes the
    # interpolation's smoothing and would be favoured by L for that alone); a
    # common shift of all volumes is a free gauge, so errors are measured after
    # removing the mean over volumes.
    truth = -torch.from_numpy(scene.drift.astype(np.float32)).cuda()

    def rms(d):
        e = d - truth
        e = e - e.mean(0, keepdim=True)
        return float(torch.sqrt((e * e).mean()))

    sh = torch.full((T, 3), 0.5, dtype=torch.float32, device="cuda")
    rms0 = rms(sh)
    L0 = float(objective(ctx.forward_shifted(cfg, xd, sh)))
    Lt = float(objective(ctx.forward_shifted(cfg, xd, truth - truth.mean(0, keepdim=True) + 0.5)))
    t0 = time.perf_counter()
    state, m = drift.refine_drift(ctx, cfg, xd, iters, start=np.full((T, 3), 0.5, np.float32), lr=0.03,
                                  stream=stream.cuda_stream)
    torch.cuda.synchronize()
    it_ms = (time.perf_counter() - t0) / max(iters, 1) * 1e3  # includes the final forward
    sh = torch.from_numpy(state.shifts).cuda()
    L1 = float(objective(m))
    # The same refinement with peak-weighted and scale-free objectives on the
    # same map (4 input voxels of border left out): whether another sharpness
    # measure turns the refinement into a drift estimator on these data.
    others = {}
    for name, kind, p in [("l2_interior", "l2", 2.0), ("l8_interior", "lp", 8.0), ("kurtosis_interior", "kurtosis", 4.0)]:
        val_o, grad_o = drift.make_objective(kind, p, border=4 * 2)
        st_o, m_o = drift.refine_drift(ctx, cfg, xd, iters, start=np.full((T, 3), 0.5, np.float32), lr=0.03,
                                       stream=stream.cuda_stream, grad_fn=grad_o)
        others[name] = {
            "objective_before": float(val_o(ctx.forward_shifted(cfg, xd, torch.full((T, 3), 0.5, device="cuda")))),
            "objective_at_true_drift": float(val_o(ctx.forward_shifted(cfg, xd, truth - truth.mean(0, keepdim=True)
                                                                       + 0.5))),
            "objective_after": float(val_o(m_o)),
            "drift_rms_error_after": rms(torch.from_numpy(st_o.shifts).cuda())}
    return {"workload": "diff: 60 x 64^3 f32 with random-walk drift, mag 2, TRAC-2 ITC0, L = -||map||",
            "voxel_volumes": units, "forward_ms": fwd_ms, "forward_adjoint_ms": fwdadj_ms,
            "fwd_adj_over_fwd": fwdadj_ms / fwd_ms, "refine_iterations": iters, "refine_ms_per_iteration": it_ms,
            "objective_before": L0, "objective_after": L1, "objective_at_true_drift": Lt,
            "drift_rms_error_before": rms0,
            "drift_rms_error_after": rms(sh), "other_objectives": others}


def measure_large(ctx, iters: int = 20, volumes=None) -> dict:
    """Large batched forward + drift refinement: 200 volumes of 256x256x128
    uint16 (8000 filament emitters, random-walk drift 0.1 voxel per volume),
    magnification 4x4x2 (1024x1024x256 map), TRAC-4 (ITC 0), intensity
    weighting; L = -||map||_2; Adam on the 200 x 3 shifts from a common
    half-voxel start. The radiality stacks of the whole series (430 GB) do not
    fit in HBM: the refinement streams the frames through HBM in batches of 25
    volumes (forward and backward carry the TRAC-4 state between batches, in as
    many z slices as one batch's scratch needs); one iteration with the map in
    z slices of all volumes is timed beside it. The input (3.4 GB) stays
    resident."""
    import torch
    from rfba_gb300 import drift, srrf, synth
    w = dict(synth.WORKLOADS["large"])
    T = volumes or w["n_vol"]
    seed = 1234 + w["index"]
    scene = synth.make_scene(seed, T, w["shape"], w["n_emitters"], w["curves"], w["drift"])
    t0 = time.perf_counter()
    x = synth.render_parallel(scene, w["shape"], seed, np.uint16)
    render_s = time.perf_counter() - t0
    cfg = srrf.Config.make(mag=(4, 4, 2), method=3, itc=0, trac_order=4, gradient_smooth=1, main_range=1,
                           x_range=1, y_range=1, z_range=1)
    xd = (torch.from_numpy(x.view(np.int16)).cuda().to(torch.int32) & 0xFFFF).to(torch.float32)
    units = xd.shape[1] * xd.shape[2] * xd.shape[3] * 32 * T
    # the plain path on the same series: GradientCalc's 16^3 blocks with a 2-voxel border
    # (GradientCalc.cpp:47-160), one launch sequence per block with its own copies
    pcfg = srrf.Config.make(mag=(4, 4, 2), method=3, itc=0, trac_order=4, gradient_smooth=1, main_range=1,
                            x_range=1, y_range=1, z_range=1, block_size=(16, 16, 16))
    gblocks, gn = srrf.blocks_gradientcalc(pcfg, x.shape)
    plain_out = np.zeros(xd.shape[1] * xd.shape[2] * xd.shape[3] * 32, np.float32)
    t0 = time.perf_counter()
    ctx.forward_blocks_plain(pcfg, x, gblocks, gn, plain_out.size, out=plain_out)
    plain_s = time.perf_counter() - t0
    del x, plain_out
    stream = torch.cuda.current_stream()
    # The forward alone (no drift correction), device input: the frames in time
    # batches of 25 volumes with the TRAC-4 window sums carried between them
    # (the automatic choice when the whole series' stacks exceed the scratch
    # budget), and the map in z slices of all 200 volumes.
    whole = {}
    for name, tbv in (("time_batches", 0), ("z_slices", -1)):
        ctx.set_time_batch(tbv)
        mm = ctx.forward(cfg, xd, stream=stream.cuda_stream)  # schedule tuning and graph capture
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        ctx.forward(cfg, xd, out=mm, stream=stream.cuda_stream)
        ev1.record(stream)
        torch.cuda.synchronize()
        vb, nb = ctx.last_time_batches()
        whole[name] = {"forward_s": ev0.elapsed_time(ev1) / 1e3, "batch_volumes": vb, "batches": nb,
                       "z_slices": ctx.last_passes(), "value": units / (ev0.elapsed_time(ev1) / 1e3)}
        del mm
    ctx.set_time_batch(0)

    objective, grad_map = drift.objective, drift.grad_map

    truth = -torch.from_numpy(scene.drift.astype(np.float32)).cuda()

    def rms(d):
        e = d - truth
        e = e - e.mean(0, keepdim=True)
        return float(torch.sqrt((e * e).mean()))

    sh = torch.full((T, 3), 0.5, dtype=torch.float32, device="cuda")
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    m = ctx.forward_shifted(cfg, xd, sh, stream=stream.cuda_stream)
    e1.record(stream)
    _, gs = ctx.backward(cfg, xd, sh, grad_map(m), stream=stream.cuda_stream)
    e2.record(stream)
    torch.cuda.synchronize()
    fwd_ms, bwd_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)
    rms0 = rms(sh)
    L0 = float(objective(m))
    del m
    # one refinement iteration with the map in z slices (forward and backward
    # each recompute the stacks of all volumes per slice), for comparison
    ctx.set_time_batch(-1)
    t0 = time.perf_counter()
    drift.refine_drift(ctx, cfg, xd, 1, start=np.full((T, 3), 0.5, np.float32), lr=0.03, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    slices_s = time.perf_counter() - t0
    # the refinement with the frames streamed through HBM in batches of 25
    # volumes: forward and backward carry the TRAC-4 state between batches
    ctx.set_time_batch(25)
    t0 = time.perf_counter()
    state, m = drift.refine_drift(ctx, cfg, xd, iters, start=np.full((T, 3), 0.5, np.float32), lr=0.03,
                                  stream=stream.cuda_stream)
    torch.cuda.synchronize()
    wall_s = time.perf_counter() - t0
    ctx.set_time_batch(0)
    sh = torch.from_numpy(state.shifts).cuda()
    return {"workload": f"large: {T} x 256x256x128 u16, 8000 filament emitters, drift 0.1/volume, mag 4x4x2, "
                        "TRAC-4 ITC0, L = -||map||, Adam on shifts from +0.5, frames in batches of 25 volumes",
            "voxel_volumes": units, "render_s": render_s, "forward_ms": fwd_ms, "backward_ms": bwd_ms,
            "forward_value": units / (fwd_ms / 1e3), "fwd_adj_over_fwd": (fwd_ms + bwd_ms) / fwd_ms,
            "refine_iterations": iters, "refine_wall_s": wall_s, "refine_s_per_iteration": wall_s / max(iters, 1),
            "refine_time_batches": 25, "refine_s_per_iteration_z_slices": slices_s,
            "objective_before": L0, "objective_after": float(objective(m)),
            "drift_rms_error_before": rms0, "drift_rms_error_after": rms(sh),
            "plain_forward_s": plain_s, "plain_blocks": gn, "forward_only": whole,
            "plain_note": "GradientCalc 16^3 blocks, border 2, one launch sequence and copy pair per block",
            "batched_forward_speedup_vs_plain": plain_s / (fwd_ms / 1e3)}


def measure_seeding(ctx, steps: int = 5) -> dict:
    """SRRF-guided spot seeding: a 29^3-voxel 3B block mask at magnification 3
    (658,503 candidate subvoxels) over a synthetic SRRF map, 100,000 spots per
    call; GPU inverse-CDF sampler (device map and voxel list) against the
    reference's rejection loop restated on the host (numpy, one core, 10,000
    spots)."""
    import torch
    from oracle import oracle as O
    rng = np.random.default_rng(12)
    mag, B = 3, 29
    m = rng.gamma(0.6, 1.0, size=(B * mag, B * mag, B * mag)).astype(np.float32)
    vox = np.array([(x, y, z) for z in range(B) for y in range(B) for x in range(B)], np.int32)
    md = torch.from_numpy(m).cuda()
    n = 100000
    ctx.seed_spots(md, vox, mag, n, seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        ctx.seed_spots(md, vox, mag, n, seed=2 + s)
    torch.cuda.synchronize()
    gpu_s = (time.perf_counter() - t0) / steps
    nc = 10000
    t0 = time.perf_counter()
    O.seed_spots_rejection(m, vox, mag, nc, np.random.default_rng(0))
    cpu_s = time.perf_counter() - t0
    return {"workload": "seeding: 29^3 mask voxels x mag 3 (658,503 candidates), 100,000 spots per call",
            "gpu_ms_per_call": gpu_s * 1e3, "gpu_spots_per_s": n / gpu_s,
            "cpu_reference_loop_spots_per_s": nc / cpu_s, "cpu_sample": f"{nc} spots, numpy, 1 core"}


def measure_combine(ctx, steps: int = 3) -> dict:
    """CombineBlock reconstruction: 50,000 localisations in a 40x40x30 image,
    zoom 10 (400x400x300 grid, 48 M voxels), the script's noise mask (r 30, rz 3,
    threshold 70) and PSF (sigma 3.5, threshold 1000); GPU against the numpy
    restatement on a 10,000-spot, zoom 5 sample."""
    from oracle import combine_oracle as C
    from rfba_gb300 import srrf
    rng = np.random.default_rng(13)
    img = (40, 40, 30)
    sp = np.empty((50000, 5))
    centres = rng.uniform(5, 25, size=(200, 3))
    k = rng.integers(0, 200, 50000)
    for a in range(3):
        sp[:, 2 + a] = np.clip(centres[k, a] + rng.normal(0, 0.4, 50000), 0, img[a] - 1)
    sp[:, 0] = 500.0
    sp[:, 1] = 1.5
    psf = srrf.combine_psf(3.5, 1000.0)
    ctx.combine_render(sp, img, 10, psf)
    t0 = time.perf_counter()
    for _ in range(steps):
        out, _ = ctx.combine_render(sp, img, 10, psf)
    gpu_s = (time.perf_counter() - t0) / steps
    small = sp[:10000]
    t0 = time.perf_counter()
    C.render(small, img, 5, psf, 30, 3, 70)
    cpu_s = time.perf_counter() - t0
    return {"workload": "combine: 50,000 spots, 40x40x30 image, zoom 10 (48 M grid voxels), PSF 3.5/1000, "
                        "mask 30/3/70", "gpu_ms_per_call": gpu_s * 1e3, "gpu_grid_voxels_per_s": out.size / gpu_s,
            "cpu_reference_s": cpu_s, "cpu_sample": "10,000 spots, zoom 5 (6 M grid voxels), numpy, 1 core",
            "cpu_grid_voxels_per_s": (40 * 5) * (40 * 5) * (30 * 5) / cpu_s}


def measure_stream(ctx, steps: int = 3, volumes=None) -> dict:
    """The forward in time batches against the one-pass forward: 100 volumes of
    64^3 uint16 (the mid workload's emitter model), mag 4x4x2 (256x256x128
    map), TRAC-4 ITC 0 with intensity weighting; batches of 25 volumes with the
    window sums carried between them (8.4 M subvoxels: 1.7 GB of stacks per
    batch and 1.3 GB of carried state) against all 100 volumes' stacks (6.7 GB)
    reduced at once; then the drift-corrected forward and its backward both
    ways (the batched backward reusing the state its forward kept), with the
    gradients compared. Device input, CUDA events."""
    import torch
    from rfba_gb300 import srrf, synth
    x, _ = synth.workload("mid", n_vol=volumes or 100, shape=(64, 64, 64))
    cfg = srrf.Config.make(**{**CFG_KW, "trac_order": 4})
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    stream = torch.cuda.current_stream()
    T = x.shape[0]
    units = 256 * 256 * 128 * T
    res, maps = {}, {}
    # time batches first: their scratch (3 GB) is all the device holds while they run
    for name, tb in (("time_batches", 25), ("one_pass", -1)):
        ctx.set_time_batch(tb)
        m = ctx.forward(cfg, xd, stream=stream.cuda_stream)
        for _ in range(2):
            ctx.forward(cfg, xd, out=m, stream=stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ctx.forward(cfg, xd, out=m, stream=stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        vb, nb = ctx.last_time_batches()
        res[name] = {"forward_ms": ms, "value": units / (ms / 1e3), "batch_volumes": vb, "batches": nb}
        maps[name] = m.cpu().numpy()
    ctx.set_time_batch(0)
    def rel_linf(got, ref):
        got, ref = np.asarray(got, np.float64), np.asarray(ref, np.float64)
        fin = np.isfinite(got) & np.isfinite(ref)
        scale = float(np.max(np.abs(ref[fin]))) if fin.any() else 0.0
        return float(np.max(np.abs(got[fin] - ref[fin]))) / scale if scale > 0 else 0.0

    rel = rel_linf(maps["time_batches"], maps["one_pass"])
    # the drift-corrected forward and its backward (L = -||map||, random shifts of
    # 0.2 voxel): in batches of 25 volumes with the carried state kept from the
    # forward for the backward, against the resident one-pass pair
    xf = xd.to(torch.int32).bitwise_and(0xFFFF).to(torch.float32)
    sh = torch.from_numpy(np.random.default_rng(7).normal(0, 0.2, size=(T, 3)).astype(np.float32)).cuda()
    fb = {}
    for name, tb in (("time_batches", 25), ("one_pass", -1)):
        ctx.set_time_batch(tb)
        for rep in range(2):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            m = ctx.forward_shifted(cfg, xf, sh, stream=stream.cuda_stream)
            e1.record(stream)
            g = torch.where(torch.isnan(m), torch.zeros_like(m),
                            -torch.nan_to_num(m) / torch.sqrt((torch.nan_to_num(m).double() ** 2).sum()).float())
            din, dsh = ctx.backward(cfg, xf, sh, g, stream=stream.cuda_stream)
            e2.record(stream)
            torch.cuda.synchronize()
        fb[name] = {"forward_ms": e0.elapsed_time(e1), "forward_backward_ms": e0.elapsed_time(e2),
                    "din": din.cpu().numpy(), "dsh": dsh.cpu().numpy()}
    ctx.set_time_batch(0)
    diff_block = {
        name: {k: v for k, v in r.items() if k not in ("din", "dsh")} for name, r in fb.items()}
    diff_block["rel_linf_din"] = rel_linf(fb["time_batches"]["din"], fb["one_pass"]["din"])
    diff_block["rel_linf_dshift"] = rel_linf(fb["time_batches"]["dsh"], fb["one_pass"]["dsh"])
    return {"workload": "stream: 100 x 64^3 u16 -> 256x256x128 map, mag 4x4x2, TRAC-4 ITC0, IW; time batches of "
                        "25 volumes vs one pass", "voxel_volumes": units, **res,
            "drift_forward_backward": diff_block,
            "time_batches_over_one_pass": res["time_batches"]["forward_ms"] / res["one_pass"]["forward_ms"],
            "nan_masks_equal": bool(np.array_equal(np.isnan(maps["one_pass"]), np.isnan(maps["time_batches"]))),
            "rel_linf_time_batches_vs_one_pass": rel}


def run_single_workload(args):
    """One of the secondary measurements alone, printed as its own JSON line."""
    import torch
    from rfba_gb300 import build as B
    B.build()
    from rfba_gb300 import srrf
    torch.cuda.set_device(0)
    ctx = srrf.Context(0)
    if args.workload == "batching":
        r = measure_batching(ctx, max(2, args.steps))
    elif args.workload == "large":
        r = measure_large(ctx, iters=args.iters, volumes=args.volumes)
    elif args.workload == "seeding":
        r = measure_seeding(ctx)
    elif args.workload == "combine":
        r = measure_combine(ctx)
    elif args.workload == "refgpu":
        r = measure_reference_gpu(ctx)
    elif args.workload == "stream":
        r = measure_stream(ctx, max(1, args.steps), volumes=args.volumes)
    elif args.workload == "threeb":
        r = measure_threeb(ctx)
        if not args.no_cpu:
            r["cpu_baseline"] = threeb_cpu_baseline(r)
    else:
        r = measure_diff(ctx, max(3, args.steps), iters=args.iters, volumes=args.volumes)
    ctx.close()
    print(json.dumps({"workload": args.workload, **r}), flush=True)


def temporal_roofline(tmp_ms, units_per_step: int, T: int, peaks: dict) -> dict:
    """HBM roofline of the temporal reduction (TRAC-2 with intensity
    weighting): per output subvoxel it must read T radiality and T intensity
    values and write the map value (the cumulant pass reads the radiality
    series a second time, mostly from L2), against the measured copy
    bandwidth."""
    if not tmp_ms:
        return {}
    ms = statistics.mean(tmp_ms)
    vox = units_per_step // T
    algo = vox * (2 * T * 4 + 4)
    hbm = float(peaks.get("hbm_gbs", 0.0)) or None
    achieved = algo / (ms / 1e3) / 1e9
    return {"kernel_ms": ms, "algorithmic_bytes": algo, "achieved_gbs": achieved, "peak_gbs": hbm,
            "frac": achieved / hbm if hbm else None, "unit": "GB/s",
            "note": "T radiality + T intensity values read and one map value written per subvoxel"}


def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from rfba_gb300 import build as B
    B.build()
    from rfba_gb300 import srrf

    x = make_input(args.volumes)
    T, D, H, W = x.shape
    cfg = srrf.Config.make(**CFG_KW)
    mx, my, mz = CFG_KW["mag"]
    out_shape = (D * mz, H * my, W * mx)
    units_per_step = out_shape[0] * out_shape[1] * out_shape[2] * T

    ctx = srrf.Context(local)
    stream = torch.cuda.current_stream()
    xd = torch.from_numpy(x.view(np.int16)).cuda()
    out = torch.empty(out_shape, dtype=torch.float32, device="cuda")

    def step():
        ctx.forward(cfg, xd, out=out, stream=stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # timed region: device time over exactly K steps
    ctx.set_timing(True)
    launches0 = ctx.timing().launches
    sampler = ClockSampler(local)
    sampler.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    rad_ms = []
    e0.record(stream)
    tmp_ms = []
    for _ in range(args.steps):
        step()
        tm = ctx.timing()
        rad_ms.append(tm.radiality_ms)
        tmp_ms.append(tm.temporal_ms)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    launches = ctx.timing().launches - launches0
    ctx.set_timing(False)
    ms = max_over_ranks(ms)
    value = whole_job_rate(units_per_step * args.steps, ws, ms / 1e3)

    # e2e: C-ABI entry point with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pinned = torch.empty(x.nbytes, dtype=torch.uint8).pin_memory()
        pinned_np = pinned.numpy().view(np.uint16).reshape(x.shape)
        pinned_np[...] = x
        outh = torch.empty(out_shape, dtype=torch.float32).pin_memory()
        outh_np = outh.numpy()
        for _ in range(max(1, args.warmup // 2)):
            ctx.forward(cfg, pinned_np, out=outh_np)
        if ws > 1:
            torch.distributed.barrier()
        e2e_step_ms = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            t1 = time.perf_counter()
            ctx.forward(cfg, pinned_np, out=outh_np)
            e2e_step_ms.append((time.perf_counter() - t1) * 1e3)
        e2e_s = time.perf_counter() - t0
        e2e_s = max_over_ranks(e2e_s)
        e2e = whole_job_rate(units_per_step * args.steps, ws, e2e_s)

    # roofline of the radiality kernel
    props = torch.cuda.get_device_properties(local)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    peak = fp32_peak_tflops(props.multi_processor_count, sm_max)
    peak_fma = srrf.probe_fp32_fma_peak(local)
    fl = algorithmic_flops_per_voxel_volume(cfg)
    rad_avg_ms = statistics.mean(rad_ms) if rad_ms else float("nan")
    achieved = fl["separable"] * units_per_step / (rad_avg_ms / 1e3) / 1e12
    traffic = None
    tf = ROOT / "profiles" / "traffic_radiality_mid.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get("bytes_per_launch")
        except Exception:
            traffic = None

    line = {
        "metric": "radiality voxel-volumes/s", "value": value, "unit": "voxel-volumes/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "mid: 100 x 128x128x64 u16 -> 512x512x128 map, mag 4x4x2, ring r 0.5, 12 axes, "
                               "smoothed gradient (ranges 1), TRAC-2 ITC0, intensity weighting",
                   "global_batch": T, "parallelism": "replicas" if ws > 1 else "single",
                   "l2": "inputs larger than L2 (210 MB input, 26.8 GB radiality/intensity stack per step)"},
        "e2e": {"value": e2e, "unit": "voxel-volumes/s", "h2d_bytes_per_step": int(x.nbytes),
                "d2h_bytes_per_step": int(np.prod(out_shape) * 4),
                "step_ms_min": min(e2e_step_ms) if e2e else None,
                "step_ms_median": statistics.median(e2e_step_ms) if e2e else None,
                "step_ms_max": max(e2e_step_ms) if e2e else None},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": "radiality_kernel<MZ=2, CZ=8, uint16, 128 threads>", "kernel_ms": rad_avg_ms,
                     "flops_per_voxel_volume": fl["separable"],
                     "peak_note": f"nominal FP32 FMA peak {props.multi_processor_count} SMs x 128 x 2 at the "
                                  f"measured max SM clock {sm_max:.0f} MHz",
                     "peak_measured_fma": peak_fma, "frac_of_measured_fma": achieved / peak_fma if peak_fma else None,
                     "peak_measured_note": "FP32 FMA chains on every SM (rfba_probe_fp32_fma_peak), measured in "
                                           "this run"},
        "direct_equivalent_tflops": fl["direct_distinct"] * units_per_step / (rad_avg_ms / 1e3) / 1e12,
        "temporal_kernel": temporal_roofline(tmp_ms, units_per_step, T, peaks),
    }
    if rank == 0 and not args.no_extras:
        line["batching"] = measure_batching(ctx, max(2, args.steps // 2))
        line["differentiation"] = measure_diff(ctx, max(3, args.steps))
        line["reference_gpu"] = measure_reference_gpu(ctx)
        line["threeb"] = measure_threeb(ctx)
        if not args.no_cpu:
            line["threeb"]["cpu_baseline"] = threeb_cpu_baseline(line["threeb"])
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(x)
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_sharded(args, make_backend=None, series=None, cfg_kw=None, block=(29, 1)):
    """--parallelism sharded: one series' block forward split across the ranks
    by rfba_gb300.shard (strong scaling: the work is fixed, the ranks share it).
    Workload: the batching series, 50 x 160^3 uint16 cut by doSplit's rule into
    216 blocks of at most 29^3 with a 1-voxel border, mag 3, TRA. Each rank
    crops its input box, runs rfba_srrf_forward_blocks on its blocks (host
    buffers: the copies are inside the timed region), and rank 0 gathers the
    packed maps (one tensor gather) and puts them back. The time is the
    slowest rank's wall time per step; the rate counts the blocks' output
    voxel-volumes once. make_backend / series / cfg_kw / block replace the
    GPU context and the workload (CPU tests). Returns (line, map) on rank 0."""
    import torch
    import torch.distributed as dist
    ws, rank, local = dist_env()
    gpu = make_backend is None
    if gpu:
        torch.cuda.set_device(local)
    if ws > 1 and not dist.is_initialized():
        dist.init_process_group("nccl" if gpu else "gloo")
    from rfba_gb300 import shard, srrf
    kw = cfg_kw or dict(mag=3, method=1, gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)
    cfg = srrf.Config.make(**kw)
    if series is None:
        from rfba_gb300 import synth
        w = dict(synth.WORKLOADS["batching"])
        seed = 1234 + w["index"]
        scene = synth.make_scene(seed, w["n_vol"], (160, 160, 160), w["n_emitters"], w["curves"], w["drift"])
        series = synth.render_parallel(scene, (160, 160, 160), seed, w["dtype"])
    x = series
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, block[0], block[1])
    units = sum(shard.block_cost(blocks[i], x.shape[0]) for i in range(n))
    backend = make_backend() if make_backend else srrf.Context(local)
    launches0 = backend.timing().launches if gpu else 0
    out = None
    for _ in range(args.warmup):
        out = shard.forward_sharded(backend, cfg, x, blocks, n, oe)
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = shard.forward_sharded(backend, cfg, x, blocks, n, oe)
    if gpu:
        torch.cuda.synchronize()
    sec = max_over_ranks(time.perf_counter() - t0)
    launches = (backend.timing().launches - launches0) if gpu else 0
    line = {"metric": "radiality voxel-volumes/s", "value": units * args.steps / sec, "unit": "voxel-volumes/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec / args.steps * 1e3,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"batching: {x.shape[0]} x {x.shape[3]}x{x.shape[2]}x{x.shape[1]} -> {n} doSplit "
                                   f"blocks ({block[0]}, border {block[1]}), mag {kw['mag']}, method {kw['method']}",
                       "parallelism": "sharded", "blocks": n,
                       "timing": "wall time per step on every rank (crop, host copies, kernels, tensor gather to "
                                 "rank 0, put-back), slowest rank"},
            "e2e": {"value": units * args.steps / sec, "unit": "voxel-volumes/s",
                    "h2d_bytes_per_step": int(x.nbytes), "d2h_bytes_per_step": int(oe * 4)},
            "gpu_launches": int(launches)}
    if gpu:
        backend.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return (line, out) if rank == 0 else (None, None)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batching (blocks vs plain) and differentiation (fwd+adj) measurements")
    ap.add_argument("--volumes", type=int, default=None,
                    help="fewer volumes than the workload's (profiling case only)")
    ap.add_argument("--iters", type=int, default=20, help="drift refinement iterations (diff workload)")
    ap.add_argument("--parallelism", default="replicas", choices=["replicas", "sharded"],
                    help="N > 1: replicas of the headline workload (default) or one batching series sharded by "
                         "blocks across the ranks")
    ap.add_argument("--workload", default="mid", choices=["mid", "batching", "diff", "large", "seeding", "combine", "refgpu", "threeb",
                             "stream"],
                    help="mid: the headline line; batching / diff: that measurement alone (one JSON line)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.parallelism == "sharded":
        run_sharded(args)
    elif args.workload != "mid":
        run_single_workload(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
