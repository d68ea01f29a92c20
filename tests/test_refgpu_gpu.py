"""The CUDA path against the reference's own CUDA kernels run on the same GPU.

baseline/refgpu.py loads kernel.cu's kernels (compiled unmodified for sm_103a)
and drives them as SRRFGradientCalcGPU (kernel.cu:560-657) and the
GradientCalc.cpp:144-160 block loop do. Both sides compute in FP32 with
different operation orders, so maps are compared by relative L-inf error with
identical NaN masks: 3e-5 for the temporal mean, TRM and TRPPM, 1e-4 for TRAC
(the tolerances of the FP64-oracle tests plus the reference's own FP32 error).
Skipped where the cubin was not built (it needs the reference sources)."""
import numpy as np
import pytest

from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

TOL = {0: 3e-5, 1: 3e-5, 2: 3e-5, 3: 1e-4}


@pytest.fixture(scope="module")
def ref():
    from baseline import refgpu
    if not refgpu.available():
        pytest.skip("reference cubin not built (baseline/build_refgpu.sh needs the reference sources)")
    r = refgpu.RefGPU(0)
    yield r
    r.close()


def _series(shape, n_vol, seed=7, emitters=30):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, n_vol, shape, emitters)
    return synth.render(scene, shape, seed, np.uint16)


SMOOTH = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)

CASES = {
    "small_tra_m2": (dict(mag=2, method=1, intensity_w=1, **SMOOTH), None),
    "trac2_itc1_m3": (dict(mag=3, method=3, itc=1, trac_order=2, intensity_w=1, **SMOOTH), ((16, 16, 14), 12)),
    "trm_central_m2": (dict(mag=2, method=0, intensity_w=1, gradient_smooth=0), ((20, 18, 16), 9)),
    "trppm_renorm_poscon_m2": (dict(mag=2, method=2, intensity_w=1, renormalize=1, remove_con=1, **SMOOTH),
                               ((18, 18, 12), 8)),
    "trac4_itc0_m2": (dict(mag=2, method=3, itc=0, trac_order=4, intensity_w=0, **SMOOTH), ((16, 16, 16), 14)),
    "trac3_itc0_m4_r07": (dict(mag=4, method=3, itc=0, trac_order=3, intensity_w=1, ring_radius=0.7,
                               axes_in_ring=4, **SMOOTH), ((12, 12, 10), 10)),
}


@pytest.mark.parametrize("case", list(CASES))
def test_whole_volume_vs_reference_kernels(ctx, ref, case):
    from rfba_gb300 import srrf, synth
    kw, shape = CASES[case]
    cfg = srrf.Config.make(**kw)
    if shape is None:
        x, _ = synth.workload("small")
    else:
        x = _series(shape[0], shape[1])
    rmap, st = ref.gradient_calc_gpu(x.astype(np.float32), cfg)
    got = ctx.forward(cfg, np.ascontiguousarray(x))
    e = assert_parity(got, rmap, TOL[kw["method"]], case + " vs reference kernels")
    print(f"[refgpu] {case}: rel L-inf {e:.2e}, reference kernels {st['kernel_ms']:.2f} ms")


def test_dosplit_blocks_vs_reference_block_loop(ctx, ref):
    """doSplit 29/1 blocks of a 40 x 40 x 30 series: the batched block path
    against the reference's per-block calls with put-back."""
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=3, method=1, intensity_w=1, **SMOOTH)
    x = _series((40, 40, 30), 6, seed=11, emitters=60)
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, 29, 1)
    assert n > 1
    got = ctx.forward_blocks(cfg, x, blocks, n, oe)
    want = np.full(oe, np.nan, np.float32)
    ref.gc_block_loop(x, cfg, blocks, n, want)
    assert_parity(got, want, TOL[1], "doSplit blocks vs reference block loop")
