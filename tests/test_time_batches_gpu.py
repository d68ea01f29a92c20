"""Forward in time batches with the temporal reduction carried between them
(temporal_stream.cu): against the one-pass reduction and the FP64 oracle, for
every method, ragged and one-volume batches, series no longer than the TRAC
order, block lists, host buffers and the automatic choice under a small
scratch budget."""
import numpy as np
import pytest

from tests.parity import assert_parity

pytestmark = pytest.mark.gpu

SHIPPED = dict(gradient_smooth=1, main_range=1, x_range=1, y_range=1, z_range=1)


def _series(seed, T, D, H, W, emitters=20):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), emitters)
    return synth.render(scene, (W, H, D), seed, np.uint16)


def _both(ctx, cfg, x, batch):
    """(one pass, batches of `batch` volumes) on the same context."""
    ctx.set_time_batch(-1)
    try:
        whole = ctx.forward(cfg, x)
        assert ctx.last_time_batches() == (0, 0)
        ctx.set_time_batch(batch)
        parts = ctx.forward(cfg, x)
        T = x.shape[0]
        if batch < T:
            assert ctx.last_time_batches() == (batch, -(-T // batch))
    finally:
        ctx.set_time_batch(0)
    return whole, parts


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("iw", [0, 1])
def test_trm_tra_trppm_bit_identical(ctx, method, iw):
    """TRM, TRA and TRPPM add the same values in the same order in batches as in
    one pass: the maps are bit-identical (kernel.cu:291-419)."""
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=method, intensity_w=iw, **SHIPPED)
    x = _series(70 + method, 23, 10, 12, 14)
    for batch in (1, 5, 22):
        whole, parts = _both(ctx, cfg, x, batch)
        assert np.array_equal(np.isnan(whole), np.isnan(parts))
        assert np.array_equal(np.nan_to_num(whole), np.nan_to_num(parts)), (method, iw, batch)


@pytest.mark.parametrize("order", [2, 3, 4])
@pytest.mark.parametrize("iw", [0, 1])
def test_trac_itc0_carried_cumulants(ctx, oracle_mod, order, iw):
    """TRAC with ITC 0 (kernel.cu:423-500): the window sums carried around the
    first batch's mean equal the one-pass reduction to rounding and the FP64
    oracle within the TRAC tolerance (1e-4 relative L-inf), with the same NaN
    mask, for batches of one volume, a ragged last batch and batches shorter
    than the order."""
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=0, trac_order=order, intensity_w=iw, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    x = _series(80 + order, 31, 10, 11, 13)
    ref = oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw))
    for batch in (1, 3, 7, 25):
        whole, parts = _both(ctx, cfg, x, batch)
        assert_parity(whole, ref, 1e-4, f"one pass TRAC-{order}")
        assert_parity(parts, ref, 1e-4, f"batches of {batch}, TRAC-{order}")
        assert_parity(parts, whole, 1e-5, f"batches of {batch} vs one pass, TRAC-{order}")


@pytest.mark.parametrize("T,order", [(2, 2), (3, 2), (4, 4), (5, 4), (1, 3)])
def test_trac_short_series(ctx, oracle_mod, T, order):
    """Series no longer than (or just past) the TRAC order: an empty or one-term
    window, in one-volume batches."""
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=0, trac_order=order, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    x = _series(90 + T, T, 6, 7, 8, emitters=4)
    whole, parts = _both(ctx, cfg, x, 1)
    ref = oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw))
    assert_parity(parts, ref, 1e-4, f"T={T} TRAC-{order}")
    assert_parity(parts, whole, 1e-5, f"T={T} TRAC-{order} vs one pass")


def test_block_list_in_batches(ctx):
    """A doSplit block list (uneven blocks, one pass each or together) in
    batches equals the one-pass block forward."""
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=3, method=3, itc=0, trac_order=3, **SHIPPED)
    x = _series(95, 17, 20, 26, 30)
    blocks, n, oe = srrf.blocks_dosplit(cfg, x.shape, (15, 15, 11), 1)
    assert n > 4
    ctx.set_time_batch(-1)
    try:
        whole = ctx.forward_blocks(cfg, x, blocks, n, oe)
        ctx.set_time_batch(4)
        parts = ctx.forward_blocks(cfg, x, blocks, n, oe)
        assert ctx.last_time_batches() == (4, 5)
    finally:
        ctx.set_time_batch(0)
    assert_parity(parts, whole, 1e-5, "block list in batches")


def test_automatic_batches_under_a_small_budget(oracle_mod):
    """With a scratch budget below the whole series' stacks but above one
    batch's stacks plus the carried state, the forward runs in batches of 25
    volumes without cutting the map; host buffers go through the captured
    graph."""
    from rfba_gb300 import srrf
    kw = dict(mag=2, method=3, itc=0, trac_order=4, **SHIPPED)
    cfg = srrf.Config.make(**kw)
    T, D, H, W = 60, 12, 14, 16
    x = _series(97, T, D, H, W)
    vox = D * H * W * 8
    fields = 38  # TRAC-4 state floats per subvoxel
    budget = vox * (25 * 8 + fields * 4) + 4096
    assert budget < vox * T * 8
    c = srrf.Context(0, budget)
    try:
        got = c.forward(cfg, x)
        assert c.last_time_batches() == (25, 3)
        again = c.forward(cfg, x)
    finally:
        c.close()
    assert np.array_equal(np.nan_to_num(got), np.nan_to_num(again))
    ref = oracle_mod.srrf_region(x.astype(np.float32), oracle_mod.make_conf(**kw))
    assert_parity(got, ref, 1e-4, "automatic batches, TRAC-4")


def test_itc1_never_batched(ctx):
    """TRAC with ITC 1 bins the whole series: a forced batch size is ignored."""
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=1, trac_order=2, **SHIPPED)
    x = _series(98, 12, 8, 9, 10)
    ctx.set_time_batch(3)
    try:
        ctx.forward(cfg, x)
        assert ctx.last_time_batches() == (0, 0)
    finally:
        ctx.set_time_batch(0)


def _drift_case(seed, T, D, H, W):
    from rfba_gb300 import synth
    scene = synth.make_scene(seed, T, (W, H, D), 10)
    x = synth.render(scene, (W, H, D), seed, np.float32)
    sh = np.random.default_rng(seed).normal(0, 0.3, size=(T, 3)).astype(np.float32)
    return x, sh


def _fwd_bwd(ctx, cfg, x, sh):
    import torch
    xd = torch.from_numpy(x).cuda()
    sd = torch.from_numpy(sh).cuda()
    m = ctx.forward_shifted(cfg, xd, sd)
    torch.cuda.synchronize()
    mh = m.cpu().numpy()
    f = np.where(np.isfinite(mh), mh, 0.0).astype(np.float64)
    g = np.where(np.isfinite(mh), -f / np.sqrt(np.sum(f * f)), 0.0).astype(np.float32)
    din, dsh = ctx.backward(cfg, xd, sd, torch.from_numpy(g).cuda())
    torch.cuda.synchronize()
    return mh, din.cpu().numpy(), dsh.cpu().numpy()


@pytest.mark.parametrize("kw,T,batch", [
    (dict(method=1, intensity_w=1), 23, 5),
    (dict(method=1, intensity_w=0, renormalize=1), 17, 4),
    (dict(method=3, itc=0, trac_order=2, intensity_w=1), 23, 5),
    (dict(method=3, itc=0, trac_order=3, intensity_w=0, remove_con=1), 19, 3),
    (dict(method=3, itc=0, trac_order=4, intensity_w=1), 26, 7),
    (dict(method=3, itc=0, trac_order=4, intensity_w=1, renormalize=1), 9, 2),
    (dict(method=3, itc=0, trac_order=4, intensity_w=0), 5, 1),
], ids=["tra_iw", "tra_renorm", "trac2_iw", "trac3_poscon", "trac4_iw", "trac4_renorm_short", "trac4_T5"])
def test_backward_in_time_batches(ctx, kw, T, batch):
    """The drift-corrected forward and its backward in time batches (forced
    size): the backward's state pass, the windows of batch + k - 1 volumes on
    either side and the carried derivatives give the gradients of the
    resident one-pass path to 1e-4 (float atomics and summation order)."""
    from tests.parity import rel_linf
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, **kw, **SHIPPED)
    x, sh = _drift_case(100 + T, T, 7, 8, 9)
    m0, din0, dsh0 = _fwd_bwd(ctx, cfg, x, sh)
    ctx.set_time_batch(batch)
    try:
        m1, din1, dsh1 = _fwd_bwd(ctx, cfg, x, sh)
    finally:
        ctx.set_time_batch(0)
    assert np.array_equal(np.isnan(m0), np.isnan(m1))
    assert rel_linf(m1, m0) < 1e-5
    assert rel_linf(din1, din0) < 1e-4, rel_linf(din1, din0)
    assert rel_linf(dsh1, dsh0) < 1e-4, rel_linf(dsh1, dsh0)


def test_backward_after_an_intervening_forward(ctx):
    """A forward on other data between a time-batched drift forward and its
    backward overwrites the carried state the backward would reuse: the
    backward must then run its own state pass and still give the resident
    path's gradients."""
    import torch
    from tests.parity import rel_linf
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=4, intensity_w=1, **SHIPPED)
    x, sh = _drift_case(131, 21, 7, 8, 9)
    other, _ = _drift_case(132, 21, 7, 8, 9)
    m0, din0, dsh0 = _fwd_bwd(ctx, cfg, x, sh)
    ctx.set_time_batch(6)
    try:
        xd = torch.from_numpy(x).cuda()
        sd = torch.from_numpy(sh).cuda()
        m1 = ctx.forward_shifted(cfg, xd, sd).cpu().numpy()
        ctx.forward_shifted(cfg, torch.from_numpy(other).cuda(), sd)  # same shape, other data
        f = np.where(np.isfinite(m1), m1, 0.0).astype(np.float64)
        g = np.where(np.isfinite(m1), -f / np.sqrt(np.sum(f * f)), 0.0).astype(np.float32)
        din1, dsh1 = ctx.backward(cfg, xd, sd, torch.from_numpy(g).cuda())
        torch.cuda.synchronize()
        din1, dsh1 = din1.cpu().numpy(), dsh1.cpu().numpy()
    finally:
        ctx.set_time_batch(0)
    assert rel_linf(m1, m0) < 1e-5
    assert rel_linf(din1, din0) < 1e-4
    assert rel_linf(dsh1, dsh0) < 1e-4


def test_batches_in_the_captured_graph_with_pinned_buffers(ctx):
    """Pinned host buffers go through the captured graph; with time batches the
    graph holds every batch's radiality launch and carry, and its replays give
    the eager map bit for bit."""
    import torch
    from rfba_gb300 import srrf
    cfg = srrf.Config.make(mag=2, method=3, itc=0, trac_order=3, intensity_w=1, **SHIPPED)
    x = _series(133, 23, 9, 10, 11)
    ctx.set_time_batch(6)
    try:
        eager = ctx.forward(cfg, x)   # pageable: eager
        assert not ctx.schedule()["graph"]
        pin_in = torch.empty(x.nbytes, dtype=torch.uint8).pin_memory().numpy().view(np.uint16).reshape(x.shape)
        pin_in[...] = x
        pin_out = torch.empty(eager.size, dtype=torch.float32).pin_memory().numpy().reshape(eager.shape)
        for _ in range(3):  # capture, then replays
            pin_out[...] = 0
            ctx.forward(cfg, pin_in, out=pin_out)
            assert ctx.schedule()["graph"] and ctx.last_time_batches() == (6, 4)
            assert np.array_equal(np.isnan(pin_out), np.isnan(eager))
            assert np.array_equal(np.nan_to_num(pin_out), np.nan_to_num(eager))
    finally:
        ctx.set_time_batch(0)
