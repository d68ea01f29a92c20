"""Drift refinement on the differentiable SRRF pair, with checkpoint and resume.

Gradient steps (Adam) on the per-volume drift shifts d_t (x, y, z in input
voxels) that minimise L = -||map||_2 over the map's finite voxels, i.e.
sharpen the SRRF map: every iteration is one drift-corrected forward
(rfba_srrf_forward_shifted: Catmull-Rom resampling of each volume by d_t, then
radiality and the temporal reduction) and its adjoint (rfba_srrf_backward:
dL/dd from the recomputed interpolated gradient field), both on the GPU. The
reference has no derivatives; this is the refinement loop the differentiable
pair exists for.

The loop state (shifts, Adam moments, iteration count) is small (T x 3 floats
three times) and can be written after every iteration; a run started with the
same arguments and `resume=True` continues from the saved iteration.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from pathlib import Path

import numpy as np


@dataclass
class DriftState:
    shifts: np.ndarray  # [T][3] float32
    m: np.ndarray       # Adam first moment
    v: np.ndarray       # Adam second moment
    it: int             # iterations done

    def save(self, path) -> None:
        """Write the state atomically (a complete file or the previous one)."""
        path = Path(path)
        tmp = path.with_name(path.name + ".tmp")
        with open(tmp, "wb") as f:
            np.savez(f, shifts=self.shifts, m=self.m, v=self.v, it=np.int64(self.it))
        os.replace(tmp, path)

    @classmethod
    def load(cls, path) -> "DriftState":
        with np.load(path) as z:
            return cls(z["shifts"].astype(np.float32), z["m"].astype(np.float32), z["v"].astype(np.float32),
                       int(z["it"]))


def objective(m):
    """L = -||map||_2 over the finite voxels (float64 sum)."""
    import torch
    f = torch.nan_to_num(m, nan=0.0).double()
    return -torch.sqrt((f * f).sum())


def grad_map(m):
    """dL/dmap of `objective`: -map / ||map|| on finite voxels, 0 on NaN."""
    import torch
    f = torch.nan_to_num(m, nan=0.0)
    return torch.where(torch.isnan(m), torch.zeros_like(m), -f / torch.sqrt((f.double() ** 2).sum()).float())


def make_objective(kind: str = "l2", p: float = 8.0, border: int = 0):
    """(value, dL/dmap) of a sharpness objective on the map's finite voxels,
    for `refine_drift`. `border` output voxels are left out on every side.

    kind "l2":       L = -||m||_2 (the default objective above).
    kind "lp":       L = -(sum max(m, 0)^p)^(1/p): the positive peaks weigh
                     more as p grows.
    kind "kurtosis": L = -N sum m^4 / (sum m^2)^2, scale-free.
    Sums are float64; the gradient is float32 with zeros on NaN voxels and in
    the border."""
    import torch

    def inner(m):
        f = torch.nan_to_num(m, nan=0.0).double()
        return f[border:-border, border:-border, border:-border] if border else f

    def value(m):
        f = inner(m)
        if kind == "l2":
            return -torch.sqrt((f * f).sum())
        if kind == "lp":
            q = torch.clamp(f, min=0.0)
            s = q.max()
            return -s * ((q / s) ** p).sum() ** (1.0 / p) if float(s.detach()) > 0 else -s
        if kind == "kurtosis":
            return -f.numel() * (f ** 4).sum() / (f * f).sum() ** 2
        raise ValueError(f"unknown objective {kind!r}")

    def grad(m):
        f = inner(m)
        if kind == "l2":
            gi = -f / torch.sqrt((f * f).sum())
        elif kind == "lp":
            q = torch.clamp(f, min=0.0)
            s = q.max()
            if float(s) > 0:
                r = q / s
                gi = -(r ** (p - 1)) * (r ** p).sum() ** (1.0 / p - 1.0)
            else:
                gi = torch.zeros_like(f)
        elif kind == "kurtosis":
            s2, s4 = (f * f).sum(), (f ** 4).sum()
            gi = -f.numel() * (4 * f ** 3 / s2 ** 2 - 4 * s4 * f / s2 ** 3)
        else:
            raise ValueError(f"unknown objective {kind!r}")
        g = torch.zeros(m.shape, dtype=torch.float64, device=m.device)
        if border:
            g[border:-border, border:-border, border:-border] = gi
        else:
            g = gi
        return torch.where(torch.isnan(m), torch.zeros_like(m), g.float()).contiguous()

    return value, grad


def refine_drift(ctx, cfg, x, iters: int, start=None, lr: float = 0.03, betas=(0.9, 0.999), eps: float = 1e-12,
                 checkpoint=None, resume: bool = False, stream=None, grad_fn=None):
    """Run Adam on the shifts until `iters` iterations are done.

    ctx: rfba_gb300.srrf.Context; cfg: Config (any temporal method);
    x: CUDA float32 tensor [T][D][H][W]; start: initial shifts [T][3] (default
    0); checkpoint: file written after every iteration; resume: continue from
    that file when it exists; grad_fn: dL/dmap of the objective minimised
    (default `grad_map`, L = -||map||_2; `make_objective` gives others).
    Returns (DriftState, map of the final shifts)."""
    import torch
    T = x.shape[0]
    dev = x.device
    if resume and checkpoint is not None and Path(checkpoint).exists():
        st = DriftState.load(checkpoint)
        if st.shifts.shape != (T, 3):
            raise ValueError(f"checkpoint holds {st.shifts.shape[0]} volumes, the series {T}")
    else:
        s0 = np.zeros((T, 3), np.float32) if start is None else np.asarray(start, np.float32).reshape(T, 3)
        st = DriftState(s0.copy(), np.zeros((T, 3), np.float32), np.zeros((T, 3), np.float32), 0)
    sh = torch.from_numpy(st.shifts).to(dev)
    mom = torch.from_numpy(st.m).to(dev)
    var = torch.from_numpy(st.v).to(dev)
    b1, b2 = betas
    s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
    m = None
    for it in range(st.it, iters):
        m = ctx.forward_shifted(cfg, x, sh, out=m, stream=s)
        _, gs = ctx.backward(cfg, x, sh, (grad_fn or grad_map)(m), stream=s)
        mom = b1 * mom + (1 - b1) * gs
        var = b2 * var + (1 - b2) * gs * gs
        sh = sh - lr * (mom / (1 - b1 ** (it + 1))) / (torch.sqrt(var / (1 - b2 ** (it + 1))) + eps)
        if checkpoint is not None:
            DriftState(sh.cpu().numpy(), mom.cpu().numpy(), var.cpu().numpy(), it + 1).save(checkpoint)
    m = ctx.forward_shifted(cfg, x, sh, out=m, stream=s)
    return DriftState(sh.cpu().numpy(), mom.cpu().numpy(), var.cpu().numpy(), max(iters, st.it)), m
