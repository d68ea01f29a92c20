"""The reference's own CUDA kernels on this GPU, driven the way the reference drives them.

What runs on the device is the reference's code: the kernels of
`RFBA Main/GradientCalc/kernel.cu` — gradKernel (kernel.cu:44-125),
calculateRadiality (kernel.cu:186-253) and the temporal kernels calculateMIP,
calculateAVE, calculatePairwiseProductSum, calculateACRF (kernel.cu:291-555) —
compiled unmodified for sm_103a by `baseline/build_refgpu.sh` into
`baseline/_ref/srrf_ref_kernel.sm_103a.cubin`. The host side is a restatement,
over the CUDA driver API (ctypes on libcuda), of `SRRFGradientCalcGPU`
(kernel.cu:560-657): every call builds the ring on the host (kernel.cu:23-33),
allocates every device buffer, copies the ring and the volume in, launches the
gradient, radiality and temporal kernels with 512-thread blocks and the
reference's grid arithmetic on the legacy default stream, frees, copies the map
out and frees the map. `gc_block_loop` restates the block loop of
GradientCalc.cpp:144-160 (host gather of one block, one call, put-back) over a
block list.

One deliberate difference, for memory safety only: the buffers that the
reference's interpolation reads get a zeroed tail. A sample exactly on the
window edge (q == dim - 1.5, kernel.cu:146 and :264) makes the reference read
tap index `dim` with weight c(-2) = 0, which for the last rows of the last time
point lies past the end of its allocation; TRAC with integrated lag times
(kernel.cu:509-520) reads up to order-1 volumes past the radiality stack when
the binned length at the first level is not a multiple of the order. With the
tails those reads stay inside the allocation and read zeros. Sizes whose `int`
products in kernel.cu:565-614 would overflow are refused.

Test and measurement infrastructure only: the library never calls this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "srrf_ref_kernel.sm_103a.cubin"
THREADS = 512  # kernel.cu:605

# C++ names of the kernels in kernel.cu (Itanium mangling of their signatures)
K_GRAD = b"_Z10gradKernelPfS_S_S_iiiiiiiii"
K_RAD = b"_Z18calculateRadialityPfS_S_ifS_iiiiiS_S_S_ii"
K_TEMPORAL = {0: b"_Z12calculateMIPPfS_S_iiiiii", 1: b"_Z12calculateAVEPfS_S_iiiiii",
              2: b"_Z27calculatePairwiseProductSumPfS_S_iiiiii", 3: b"_Z13calculateACRFPfS_S_iiiiiiii"}


def available() -> bool:
    return CUBIN.exists()


def build(reference_root: str | None = None) -> Path | None:
    """Compile the cubin where the reference sources are present (found by
    oracle.refroot.reference_root: RFBA_REFERENCE_ROOT, then the argument)."""
    from oracle.refroot import reference_root as _root
    reference_root = _root(reference_root)
    if os.path.isdir(reference_root):
        subprocess.run(["bash", str(HERE / "build_refgpu.sh"), reference_root], check=True)
    return CUBIN if CUBIN.exists() else None


def ring(radius: float, n: int):
    """kernel.cu:23-33 on the host: float angle step from PI = 3.141592654f
    (kernel.cu:17), libm's float sin/cos, (r * sin) * cos association."""
    libm = ctypes.CDLL("libm.so.6")
    libm.sinf.restype = libm.cosf.restype = ctypes.c_float
    libm.sinf.argtypes = libm.cosf.argtypes = [ctypes.c_float]
    f = np.float32
    step = f(f(3.141592654) * f(2.0)) / f(n)
    rx, ry, rz = (np.empty(n * n, np.float32) for _ in range(3))
    r = f(radius)
    for i in range(n):
        a = f(step * f(i))
        s1, c1 = f(libm.sinf(a)), f(libm.cosf(a))
        for j in range(n):
            b = f(step * f(j))
            k = i * n + j
            rx[k] = f(r * s1) * f(libm.cosf(b))
            ry[k] = f(r * s1) * f(libm.sinf(b))
            rz[k] = f(r * c1)
    return rx, ry, rz


def _conf(cfg) -> dict:
    """The SRRFConf fields (kernel.cuh:3-24) from a Config of the extended API."""
    mag = [int(v) for v in cfg.mag]
    if len(set(mag)) != 1:
        raise ValueError("the reference has one magnification for all axes")
    return dict(r=float(cfg.ring_radius), mag=mag[0], n=2 * int(cfg.axes_in_ring), mR=int(cfg.main_range),
                xR=int(cfg.x_range), yR=int(cfg.y_range), zR=int(cfg.z_range), method=int(cfg.method),
                itc=int(cfg.itc), order=int(cfg.trac_order), rc=int(cfg.remove_con), renorm=int(cfg.renormalize),
                smooth=int(cfg.gradient_smooth), iw=int(cfg.intensity_w))


class RefGPU:
    """The reference's kernels loaded into the primary context of one device."""

    def __init__(self, device: int = 0, cubin: Path = CUBIN):
        if not Path(cubin).exists():
            raise FileNotFoundError(f"{cubin} not built (baseline/build_refgpu.sh needs the reference sources)")
        cu = ctypes.CDLL("libcuda.so.1")
        self._cu = cu
        cu.cuGetErrorString.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p)]
        cu.cuMemAlloc_v2.argtypes = [ctypes.POINTER(ctypes.c_uint64), ctypes.c_size_t]
        cu.cuMemFree_v2.argtypes = [ctypes.c_uint64]
        cu.cuMemcpyHtoD_v2.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_size_t]
        cu.cuMemcpyDtoH_v2.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_size_t]
        cu.cuMemsetD8_v2.argtypes = [ctypes.c_uint64, ctypes.c_ubyte, ctypes.c_size_t]
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        cu.cuEventRecord.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        cu.cuEventElapsedTime_v2.argtypes = [ctypes.POINTER(ctypes.c_float), ctypes.c_void_p, ctypes.c_void_p]
        self._ck(cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._ck(cu.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
        self._ctx = ctypes.c_void_p()
        self._ck(cu.cuDevicePrimaryCtxRetain(ctypes.byref(self._ctx), dev), "cuDevicePrimaryCtxRetain")
        self._dev = dev
        self._ck(cu.cuCtxSetCurrent(self._ctx), "cuCtxSetCurrent")
        self._mod = ctypes.c_void_p()
        self._ck(cu.cuModuleLoad(ctypes.byref(self._mod), str(cubin).encode()), "cuModuleLoad")
        self._fn = {}
        for key, name in [("grad", K_GRAD), ("rad", K_RAD)] + list(K_TEMPORAL.items()):
            f = ctypes.c_void_p()
            self._ck(cu.cuModuleGetFunction(ctypes.byref(f), self._mod, name), "cuModuleGetFunction " + name.decode())
            self._fn[key] = f
        self._ev = []
        for _ in range(6):
            e = ctypes.c_void_p()
            self._ck(cu.cuEventCreate(ctypes.byref(e), 0), "cuEventCreate")
            self._ev.append(e)

    def close(self):
        if getattr(self, "_mod", None):
            self._cu.cuCtxSetCurrent(self._ctx)
            for e in self._ev:
                self._cu.cuEventDestroy_v2(e)
            self._cu.cuModuleUnload(self._mod)
            self._cu.cuDevicePrimaryCtxRelease_v2(self._dev)
            self._mod = None

    def _ck(self, rc: int, what: str):
        if rc != 0:
            s = ctypes.c_char_p()
            self._cu.cuGetErrorString(rc, ctypes.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")

    def _alloc(self, nbytes: int) -> ctypes.c_uint64:
        p = ctypes.c_uint64()
        self._ck(self._cu.cuMemAlloc_v2(ctypes.byref(p), nbytes), "cuMemAlloc")
        return p

    def _launch(self, key, grid: int, args):
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self._ck(self._cu.cuLaunchKernel(self._fn[key], grid, 1, 1, THREADS, 1, 1, 0, None, params, None),
                 "cuLaunchKernel")

    def gradient_calc_gpu(self, img: np.ndarray, cfg):
        """SRRFGradientCalcGPU (kernel.cu:560-657) on img [T][D][H][W] float32.
        Returns (map [D*mag][H*mag][W*mag] float32, {"kernel_ms", "call_ms"}):
        kernel_ms is the device time of the three kernels (events around each),
        call_ms the host time of the whole synchronous call."""
        c = _conf(cfg)
        img = np.ascontiguousarray(img, np.float32)
        T, D, H, W = img.shape
        m, n = c["mag"], c["n"]
        whd = W * H * D
        whdt = whd * T
        m3 = m * m * m
        if whdt * m3 >= 2 ** 31:
            raise ValueError("the reference's int index arithmetic (kernel.cu:565-614) overflows at this size")
        rx, ry, rz = ring(c["r"], n)
        tail = (H + 1) * W + 64
        rad_tail = c["order"] * whd * m3 if (c["method"] == 3 and c["itc"] == 1) else 0
        cu, I, F, P = self._cu, ctypes.c_int, ctypes.c_float, ctypes.c_uint64
        self._ck(cu.cuCtxSetCurrent(self._ctx), "cuCtxSetCurrent")
        t0 = time.perf_counter()
        ringd = []
        for a in (rx, ry, rz):
            p = self._alloc(a.nbytes)
            self._ck(cu.cuMemcpyHtoD_v2(p, a.ctypes.data, a.nbytes), "HtoD ring")
            ringd.append(p)
        imgd = self._alloc((whdt + tail) * 4)
        self._ck(cu.cuMemsetD8_v2(imgd, 0, (whdt + tail) * 4), "memset")
        self._ck(cu.cuMemcpyHtoD_v2(imgd, img.ctypes.data, whdt * 4), "HtoD image")
        G = []
        for _ in range(3):
            p = self._alloc((whdt + tail) * 4)
            self._ck(cu.cuMemsetD8_v2(p, 0, (whdt + tail) * 4), "memset")
            G.append(p)
        ev = self._ev
        cu.cuEventRecord(ev[0], None)
        self._launch("grad", whdt // THREADS + 1,
                     [P(imgd.value), P(G[0].value), P(G[1].value), P(G[2].value), I(W), I(H), I(D), I(T),
                      I(c["smooth"]), I(c["mR"]), I(c["xR"]), I(c["yR"]), I(c["zR"])])
        cu.cuEventRecord(ev[1], None)
        radd = self._alloc((whdt * m3 + rad_tail) * 4)
        self._ck(cu.cuMemsetD8_v2(radd, 0, (whdt * m3 + rad_tail) * 4), "memset")
        grid = whd * m3 // THREADS + 1
        cu.cuEventRecord(ev[2], None)
        self._launch("rad", grid,
                     [P(ringd[0].value), P(ringd[1].value), P(ringd[2].value), I(n), F(c["r"]), P(radd.value),
                      I(W * m), I(H * m), I(D * m), I(T), I(m), P(G[0].value), P(G[1].value), P(G[2].value),
                      I(c["renorm"]), I(c["rc"])])
        cu.cuEventRecord(ev[3], None)
        srrfd = self._alloc(whd * m3 * 4)
        self._ck(cu.cuMemsetD8_v2(srrfd, 0, whd * m3 * 4), "memset")
        targs = [P(srrfd.value), P(radd.value), P(imgd.value), I(W * m), I(H * m), I(D * m), I(T), I(m), I(c["iw"])]
        if c["method"] == 3:
            targs += [I(c["itc"]), I(c["order"])]
        cu.cuEventRecord(ev[4], None)
        self._launch(c["method"], grid, targs)
        cu.cuEventRecord(ev[5], None)
        for p in ringd + [imgd] + G + [radd]:
            self._ck(cu.cuMemFree_v2(p), "cuMemFree")
        out = np.empty((D * m, H * m, W * m), np.float32)
        self._ck(cu.cuMemcpyDtoH_v2(out.ctypes.data, srrfd, out.nbytes), "DtoH map")
        self._ck(cu.cuMemFree_v2(srrfd), "cuMemFree")
        call_ms = (time.perf_counter() - t0) * 1e3
        self._ck(cu.cuCtxSynchronize(), "cuCtxSynchronize")
        kms = 0.0
        for a, b in ((0, 1), (2, 3), (4, 5)):
            ms = ctypes.c_float()
            self._ck(cu.cuEventElapsedTime_v2(ctypes.byref(ms), ev[a], ev[b]), "cuEventElapsedTime")
            kms += ms.value
        return out, {"kernel_ms": kms, "call_ms": call_ms}

    def gc_block_loop(self, x: np.ndarray, cfg, blocks, nblocks: int, out: np.ndarray):
        """GradientCalc.cpp:144-160 over a block list: for each block, a host
        copy of its sub-volume as float32 (doSplit), one gradient_calc_gpu call,
        and the put-back of its [lo, hi) region through the block's output
        offset and strides. Returns {"kernel_ms", "call_ms", "wall_ms"}."""
        kms = cms = 0.0
        t0 = time.perf_counter()
        for i in range(nblocks):
            b = blocks[i]
            (ox, oy, oz), (sx, sy, sz) = tuple(b.origin), tuple(b.size)
            sub = np.ascontiguousarray(x[:, oz:oz + sz, oy:oy + sy, ox:ox + sx], dtype=np.float32)
            mp, st = self.gradient_calc_gpu(sub, cfg)
            kms += st["kernel_ms"]
            cms += st["call_ms"]
            lo, hi = tuple(b.lo), tuple(b.hi)
            reg = mp[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]]
            zz, yy, xx = np.meshgrid(np.arange(hi[2] - lo[2]), np.arange(hi[1] - lo[1]), np.arange(hi[0] - lo[0]),
                                     indexing="ij")
            idx = b.out_offset + xx * b.out_stride[0] + yy * b.out_stride[1] + zz * b.out_stride[2]
            out[idx.ravel()] = reg.ravel()
        return {"kernel_ms": kms, "call_ms": cms, "wall_ms": (time.perf_counter() - t0) * 1e3}
