"""One series' SRRF work split across processes, one GPU each.

Output voxels are independent given their input halo, so the work partitions
without exchanging map data:

- Map blocks. The block list of a forward (GradientCalc.cpp:47-116's split or
  doSplit.m's) is dealt out longest first, each block to the rank with the
  least work so far (work = region voxels x volumes). Every rank computes its
  blocks from its own input box (the union of its blocks' sub-volumes, halos
  included) into one packed buffer; rank 0 gathers the buffers (one tensor
  gather) and puts each block's region back where the original block list
  placed it. No collective touches the maps, only that gather.
- Drift refinement (rfba_gb300.drift's Adam loop on the per-volume shifts).
  The fine map is cut into z slabs, one per rank. Each rank runs the region
  forward and region adjoint (rfba_srrf_forward_shifted_region /
  rfba_srrf_backward_region) on its slab. Per iteration, two all-reduces make
  every rank take the same step: one of the slab's sum of squares (the
  objective's norm), one of dL/dshifts (T x 3 floats).

For the drift refinement every rank holds the whole input series: the drift
resampling moves voxels along all three axes, so a slab's input halo depends
on the shifts.

`backend` is anything with the rfba_gb300.srrf.Context methods used here
(forward_blocks, forward_shifted_region, backward_region); the processes
share a torch.distributed group (NCCL on GPUs, gloo elsewhere).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from .drift import DriftState
from .srrf import Block


def _rank_world(group=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_rank(group), dist.get_world_size(group)
    return 0, 1


def block_cost(b: Block, T: int) -> int:
    """Work of one block: its magnified region's voxels times the volumes."""
    n = 1
    for a in range(3):
        n *= max(0, b.hi[a] - b.lo[a])
    return n * T


def balance(costs, world: int):
    """Longest-first greedy: each item, largest first, goes to the rank with
    the least work so far (the lowest rank on a tie). Returns one index list
    per rank, each in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0] * world
    parts = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(world), key=lambda r: (load[r], r))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def repack(blocks, idx):
    """The blocks `idx` of a list with each region written packed [z][y][x],
    one after another. Returns (Block array, count, packed elements)."""
    sub = (Block * max(len(idx), 1))()
    off = 0
    for k, i in enumerate(idx):
        b = blocks[i]
        ctypes.memmove(ctypes.byref(sub[k]), ctypes.byref(b), ctypes.sizeof(Block))
        nx, ny, nz = (b.hi[a] - b.lo[a] for a in range(3))
        sub[k].out_offset = off
        sub[k].out_stride[0], sub[k].out_stride[1], sub[k].out_stride[2] = 1, nx, nx * ny
        off += nx * ny * nz
    return sub, len(idx), off


def put_back(out: np.ndarray, blocks, idx, packed: np.ndarray) -> None:
    """Write a rank's packed regions (from `repack(blocks, idx)`) into the flat
    output `out` at the offsets and strides of the original block list."""
    packed = np.asarray(packed).reshape(-1)
    off = 0
    for i in idx:
        b = blocks[i]
        nx, ny, nz = (b.hi[a] - b.lo[a] for a in range(3))
        n = nx * ny * nz
        s0, s1, s2 = b.out_stride[0], b.out_stride[1], b.out_stride[2]
        dst = (b.out_offset + np.arange(nz, dtype=np.int64)[:, None, None] * s2 +
               np.arange(ny, dtype=np.int64)[None, :, None] * s1 + np.arange(nx, dtype=np.int64)[None, None, :] * s0)
        out[dst.reshape(-1)] = packed[off:off + n]
        off += n


def input_box(blocks, idx):
    """The input box [lo, hi) (x, y, z) that the blocks `idx` read: the union of
    their sub-volumes, halos included (a block reads nothing outside its own
    origin and size)."""
    lo = [min(blocks[i].origin[a] for i in idx) for a in range(3)]
    hi = [max(blocks[i].origin[a] + blocks[i].size[a] for i in idx) for a in range(3)]
    return lo, hi


def crop(x, blocks, idx):
    """This rank's input: the series cut to input_box (a contiguous copy) and
    the blocks' Block array with origins relative to it, packed outputs."""
    lo, hi = input_box(blocks, idx)
    xs = x[:, lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
    xs = np.ascontiguousarray(xs) if isinstance(x, np.ndarray) else xs.contiguous()
    sub, n, elems = repack(blocks, idx)
    for k in range(n):
        for a in range(3):
            sub[k].origin[a] -= lo[a]
    return xs, sub, n, elems


def forward_local(backend, cfg, x, blocks, nblocks: int, rank: int, world: int, stream=None):
    """This rank's share of a block forward: (block indices, packed regions).
    Only the input box of the rank's blocks is handed to the backend, so a rank
    holds its slab and halo, not the whole series."""
    T = x.shape[0]
    idx = balance([block_cost(blocks[i], T) for i in range(nblocks)], world)[rank]
    if not idx:
        return idx, np.zeros(0, np.float32)
    xs, sub, n, elems = crop(x, blocks, idx)
    packed = backend.forward_blocks(cfg, xs, sub, n, elems, stream=stream)
    if not isinstance(packed, np.ndarray):
        packed = packed.cpu().numpy()
    return idx, packed


def gather_packed(packed: np.ndarray, group=None):
    """Every rank's packed float32 buffer on rank 0 (a list in rank order; None
    on the other ranks), as tensors: the lengths first (one all-gather of an
    int64), then one gather of the buffers padded to the longest. Tensors live
    where the backend wants them (CUDA for NCCL); the values travel bit for
    bit, NaN included."""
    import torch
    import torch.distributed as dist
    rank, world = _rank_world(group)
    packed = np.ascontiguousarray(packed, np.float32).reshape(-1)
    if world == 1:
        return [packed]
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    n = torch.tensor([packed.size], dtype=torch.int64, device=dev)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(v.item()) for v in sizes]
    m = max(max(sizes), 1)
    buf = torch.zeros(m, dtype=torch.float32, device=dev)
    if packed.size:
        buf[:packed.size] = torch.from_numpy(packed).to(dev)
    root = dist.get_global_rank(group, 0) if group is not None else 0
    bufs = [torch.empty(m, dtype=torch.float32, device=dev) for _ in range(world)] if rank == 0 else None
    dist.gather(buf, bufs, dst=root, group=group)
    if rank != 0:
        return None
    return [b[:k].cpu().numpy() for b, k in zip(bufs, sizes)]


def forward_sharded(backend, cfg, x, blocks, nblocks: int, out_elems: int, group=None, stream=None):
    """Block forward split across the group's ranks; rank 0 returns the flat
    output (as one process's rfba_srrf_forward_blocks writes it, starting from
    zeros), the other ranks None. The ranks' block lists follow from `balance`
    on every rank alike, so only the packed maps travel (gather_packed)."""
    rank, world = _rank_world(group)
    T = x.shape[0]
    parts = balance([block_cost(blocks[i], T) for i in range(nblocks)], world)
    idx, packed = forward_local(backend, cfg, x, blocks, nblocks, rank, world, stream)
    maps = gather_packed(packed, group)
    if rank != 0:
        return None
    out = np.zeros(out_elems, np.float32)
    for r in range(world):
        put_back(out, blocks, parts[r], maps[r])
    return out


def z_slabs(nz: int, world: int):
    """[z0, z1) per rank covering 0..nz, sizes differing by at most one."""
    q, r = divmod(nz, world)
    edges = [0]
    for k in range(world):
        edges.append(edges[-1] + q + (1 if k < r else 0))
    return [(edges[k], edges[k + 1]) for k in range(world)]


def _all_reduce_sum(t, group=None):
    """Sum over the group; gloo groups reduce a host copy."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return t
    if t.is_cuda and dist.get_backend(group) != "nccl":
        h = t.cpu()
        dist.all_reduce(h, group=group)
        return h.to(t.device)
    dist.all_reduce(t, group=group)
    return t


def refine_drift_sharded(backend, cfg, x, iters: int, start=None, lr: float = 0.03, betas=(0.9, 0.999),
                         eps: float = 1e-12, checkpoint=None, resume: bool = False, group=None, stream=None):
    """rfba_gb300.drift.refine_drift with the map cut into z slabs across the
    group's ranks. Every rank ends with the same shifts; rank 0 writes the
    checkpoint. Returns (DriftState, this rank's slab of the final map
    [z1-z0][H*mag][W*mag] or None when the slab is empty (more ranks than map
    planes), (z0, z1))."""
    import torch
    rank, world = _rank_world(group)
    T, D, H, W = x.shape
    dev = x.device
    z0, z1 = z_slabs(D * cfg.mag[2], world)[rank]
    lo, hi = (0, 0, z0), (W * cfg.mag[0], H * cfg.mag[1], z1)
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
    if stream is None and x.is_cuda:
        stream = torch.cuda.current_stream().cuda_stream
    m = None
    for it in range(st.it, iters):
        if z1 > z0:
            m = backend.forward_shifted_region(cfg, x, sh, lo, hi, out=m, stream=stream)
            f = torch.nan_to_num(m, nan=0.0)
            ss = (f.double() ** 2).sum().reshape(1)
        else:
            ss = torch.zeros(1, dtype=torch.float64, device=dev)
        ss = _all_reduce_sum(ss, group)
        if z1 > z0:
            g = torch.where(torch.isnan(m), torch.zeros_like(m), -f / torch.sqrt(ss[0]).float())
            _, gs = backend.backward_region(cfg, x, sh, lo, hi, g, stream=stream)
        else:
            gs = torch.zeros_like(sh)
        gs = _all_reduce_sum(gs.contiguous(), group)
        mom = b1 * mom + (1 - b1) * gs
        var = b2 * var + (1 - b2) * gs * gs
        sh = sh - lr * (mom / (1 - b1 ** (it + 1))) / (torch.sqrt(var / (1 - b2 ** (it + 1))) + eps)
        if checkpoint is not None and rank == 0:
            DriftState(sh.cpu().numpy(), mom.cpu().numpy(), var.cpu().numpy(), it + 1).save(checkpoint)
    if z1 > z0:
        m = backend.forward_shifted_region(cfg, x, sh, lo, hi, out=m, stream=stream)
    return DriftState(sh.cpu().numpy(), mom.cpu().numpy(), var.cpu().numpy(), max(iters, st.it)), m, (z0, z1)
