"""The forward entry point that allocates no device memory.

rfba_srrf_forward_static_scratch is for callers that cannot call cudaMalloc
where they need a map (an acquisition loop that must not stall on cudaMalloc's
device-wide synchronisation, a host whose device memory belongs to its own
pool, a plugin environment that forbids device allocation): it keeps every
temporary in one fixed device array inside the library. These tests call it
through the C-ABI on device buffers and compare its maps with the allocating
entry point's on two calls in a row, with different inputs and methods, so a
stale work counter or stale stack contents from the first call would show in
the second. This file is collected last so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

from tests.parity import assert_parity, tol_for

pytestmark = pytest.mark.gpu


def _entry():
    from rfba_gb300 import srrf
    L = srrf.lib()
    fn = L.rfba_srrf_forward_static_scratch
    fn.argtypes = [ctypes.POINTER(srrf.Config), ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                   ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def _series(seed, T, D, H, W):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 15)
    return synth.render(scene, (W, H, D), seed, np.uint16)


def test_static_scratch_matches_allocating_forward_twice():
    import torch
    from rfba_gb300 import srrf

    fn = _entry()
    ctx = srrf.Context(0)
    try:
        cases = [
            (dict(mag=2, method=1, gradient_smooth=1, x_range=1, y_range=1, z_range=1), (8, 11, 12, 13), 31),
            (dict(mag=(4, 4, 2), method=3, itc=1, trac_order=2, gradient_smooth=1, x_range=1, y_range=1,
                  z_range=1), (12, 9, 10, 11), 32),
        ]
        stream = torch.cuda.current_stream()
        for kw, shape, seed in cases:
            cfg = srrf.Config.make(**kw)
            x = _series(seed, *shape)
            xd = torch.from_numpy(x.view(np.int16)).cuda()
            ref = ctx.forward(cfg, xd)
            torch.cuda.synchronize()
            T, D, H, W = shape
            dims = (ctypes.c_int * 4)(W, H, D, T)
            out = torch.full(tuple(ref.shape), float("nan"), dtype=torch.float32, device="cuda")
            rc = fn(ctypes.byref(cfg), ctypes.c_void_p(xd.data_ptr()), srrf.RFBA_U16, dims,
                    ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
            assert rc == 0, srrf.last_error()
            torch.cuda.synchronize()
            assert_parity(out.cpu().numpy(), ref.cpu().numpy(), tol_for(cfg.method), f"static scratch {kw}")
    finally:
        ctx.close()


def test_static_scratch_rejects_oversize_volume():
    import torch
    from rfba_gb300 import srrf

    fn = _entry()
    cfg = srrf.Config.make(mag=2, method=1)
    # 64 x 64 x 64 input at mag 2 over 20 volumes: 2.1e6 subvoxels x 20 x 8 bytes = 336 MB > 128 MiB
    T, D, H, W = 20, 64, 64, 64
    xd = torch.zeros((T, D, H, W), dtype=torch.int16, device="cuda")
    out = torch.empty((D * 2, H * 2, W * 2), dtype=torch.float32, device="cuda")
    dims = (ctypes.c_int * 4)(W, H, D, T)
    rc = fn(ctypes.byref(cfg), ctypes.c_void_p(xd.data_ptr()), srrf.RFBA_U16, dims, ctypes.c_void_p(out.data_ptr()),
            None)
    assert rc == -2  # RFBA_ERR_UNSUPPORTED
    assert "static scratch" in srrf.last_error()


def test_static_scratch_rejects_host_pointers():
    from rfba_gb300 import srrf

    fn = _entry()
    cfg = srrf.Config.make(mag=2, method=1)
    x = np.zeros((2, 8, 8, 8), np.uint16)
    out = np.zeros((16, 16, 16), np.float32)
    dims = (ctypes.c_int * 4)(8, 8, 8, 2)
    rc = fn(ctypes.byref(cfg), ctypes.c_void_p(x.ctypes.data), srrf.RFBA_U16, dims, ctypes.c_void_p(out.ctypes.data),
            None)
    assert rc == -1
    assert "device pointers" in srrf.last_error()
