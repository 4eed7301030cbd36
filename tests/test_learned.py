"""Learned minimum variance: the network's kernels against the CPU oracle
(forward, gradients, Adam), the feature kernel and the Capon-weight export
against the C oracle's restatement, the gate and fallback, and what training
gains over the same combiner with uniform weights.

The network and the learned combiner have no counterpart in the reference;
the oracle for the network is oracle/mlp_oracle.py and for the features and
weights oracle/usx_oracle_impl.inc (orc_mv_training_pairs), whose minimum
variance reproduces the reference's golden frames bit for bit."""

from __future__ import annotations

import numpy as np
import pytest

from gold import BF_CASES, rel_l2, sim_setup, txset
from oracle import mlp_oracle as MO
from oracle import oracle as O

DIMS = (256, 256, 256, 256, 128)


# ------------------------------------------------------------------ CPU

def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1e-3, 65504.0], np.float32)
    got = MO.bf16(x)
    assert got[0] == 1.0
    assert got[1] == 1.0                      # tie -> even mantissa
    assert got[2] == 1.0 + 2.0 ** -6          # tie -> even (up)
    assert got[3] == -2.5
    assert abs(got[4] - 1e-3) / 1e-3 < 2.0 ** -8
    assert got[5] == 65536.0


def test_mlp_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    dims = (6, 10, 8, 4)
    n = sum(a * b + b for a, b in zip(dims[:-1], dims[1:]))
    p = rng.standard_normal(n) * 0.5
    x = rng.standard_normal((7, dims[0]))
    t = rng.standard_normal((7, dims[-1]))
    m = (rng.random((7, dims[-1])) > 0.3).astype(np.float64)
    _, g = MO.backward(p, dims, x, t, m, quantize=False)
    fd = np.empty(n)
    h = 1e-6
    for i in range(n):
        e = np.zeros(n)
        e[i] = h
        fd[i] = (MO.loss(p + e, dims, x, t, m) - MO.loss(p - e, dims, x, t, m)) / (2 * h)
    assert np.max(np.abs(fd - g)) < 1e-7 * max(1.0, np.max(np.abs(g)))


def test_lmv_output_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(8)
    rows = 3
    y = rng.standard_normal((rows, 128)) + np.tile([1.0, 0.0], 64)
    t = rng.standard_normal((rows, 128)) + np.tile([1.0, 0.0], 64)
    x = rng.standard_normal((rows, 256))
    L = np.array([5, 17, 64])
    mask = (np.arange(128)[None, :] // 2 < L[:, None]).astype(np.float64)
    loss, g = MO.lmv_output_loss(y, t, mask, x, 0.1)
    h = 1e-6
    for r in range(rows):
        for k in (0, 1, 8, 9, 2 * L[r] - 1, 2 * L[r] - 2):
            e = np.zeros_like(y)
            e[r, k] = h
            fd = (MO.lmv_output_loss(y + e, t, mask, x, 0.1)[0] - MO.lmv_output_loss(y - e, t, mask, x, 0.1)[0]) / (2 * h)
            assert abs(fd - g[r, k]) < 1e-6 * max(1.0, abs(fd))
    assert np.all(g[mask == 0] == 0)


def test_lmv_subspace_loss_gradient_matches_finite_differences():
    rng = np.random.default_rng(9)
    rows = 3
    y = rng.standard_normal((rows, 128))
    t = rng.standard_normal((rows, 128))
    L = np.array([3, 17, 64])
    mask = (np.arange(128)[None, :] // 2 < L[:, None]).astype(np.float64)
    loss, g = MO.lmv_subspace_loss(y, t, mask, 0.1)
    assert loss > 0
    h = 1e-6
    for r in range(rows):
        for k in (0, 1, 4, 5, 2 * L[r] - 1, 2 * L[r] - 2):
            e = np.zeros_like(y)
            e[r, k] = h
            fd = (MO.lmv_subspace_loss(y + e, t, mask, 0.1)[0] - MO.lmv_subspace_loss(y - e, t, mask, 0.1)[0]) / (2 * h)
            assert abs(fd - g[r, k]) < 1e-6 * max(1.0, abs(fd))
    assert np.all(g[mask == 0] == 0)
    # Scale and phase of the complement direction do not matter: a target
    # equal to (1 + 2j) times the prediction has zero direction loss.
    w = y[:, 0::2] + 1j * y[:, 1::2]
    t2 = np.zeros_like(y)
    t2[:, 0::2], t2[:, 1::2] = ((1 + 2j) * w).real, ((1 + 2j) * w).imag
    l2, _ = MO.lmv_subspace_loss(y, t2, mask, 0.0)
    assert l2 < 1e-12


def test_weights_file_roundtrip(tmp_path):
    from usx import learned
    rng = np.random.default_rng(0)
    n = sum(a * b + b for a, b in zip(DIMS[:-1], DIMS[1:]))
    p = rng.standard_normal(n).astype(np.float32)
    f = tmp_path / "w.bin"
    learned.save_weights(f, DIMS, p)
    dims, q = learned.load_weights(f)
    assert dims == DIMS and np.array_equal(p, q)
    f.write_bytes(b"nonsense" + f.read_bytes()[8:])
    with pytest.raises(ValueError):
        learned.load_weights(f)


def test_mode_selection_respects_the_fallback_budget():
    """The shipped setting is the lowest-fallback mode that meets the quality
    bar within the fallback budget, else the mode closest to the bar within
    it; the mode that meets the bar at any cost is recorded beside it."""
    from usx import learned
    M = learned.Mode

    def res(fb, dg, lat, ax):
        return {"fallback_rate": fb, "gcnr": {"max_abs_delta": dg},
                "lateral_fwhm_mm": {"max_rel_delta": lat}, "axial_fwhm_mm": {"max_rel_delta": ax}}
    modes = [M(), M(level=10.0), M(level=3.0, share=0.02), M(use_net=False)]
    results = {modes[0].label: res(0.0, 0.008, 0.80, 0.018), modes[1].label: res(0.055, 0.008, 0.027, 0.018),
               modes[2].label: res(0.70, 0.008, 0.0, 0.005), modes[3].label: res(0.0, 0.014, 0.09, 0.80)}
    chosen, ok = learned.choose_mode(results, modes)
    assert chosen == modes[1] and not ok            # the bar is met only beyond the budget
    assert learned.at_bar_mode(results, modes) == modes[2]
    chosen, ok = learned.choose_mode(results, modes, max_fallback=0.8)
    assert chosen == modes[2] and ok
    assert M(level=10.0, window=(1, 2)).label.endswith(",level=10,win=1x2")
    assert M(level=10.0).label == "gate=inf,share=inf,level=10"


def _golden_mv_case(golden, name="mv"):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    return g, s, pr, med, acq


def test_oracle_training_pairs_reproduce_the_reference_frame(oracle, golden):
    """The training export rides on the oracle's minimum variance, which is
    the reference's to the bit; the exported weights are L w / sum(w)."""
    g, s, pr, med, acq = _golden_mv_case(golden)
    cd = O.channel_desc(pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    n0, n1 = len(g["ax0"]), len(g["ax1"])
    fr, feat, w, valid = oracle.mv_training_pairs(cd, g["iq"], g["pts"], n0, n1, O.bf_config(**BF_CASES["mv"]))
    assert np.array_equal(fr.astype(np.complex64), g["bf_mv"])
    ok = valid == 1
    assert ok.mean() > 0.9
    L = np.round(feat[:, 0] * 64).astype(int)
    wc = w[:, 0::2] + 1j * w[:, 1::2]
    assert np.max(np.abs(wc[ok].sum(1) / L[ok] - 1)) < 1e-5
    for r in np.nonzero(ok)[0][:50]:
        assert np.all(wc[r, L[r]:] == 0) and np.all(feat[r, 2 * L[r]:128] == 0)
    assert np.all(feat[~ok & (L == 0)] == 0)


def test_oracle_subspace_with_full_span_is_exact_mv(oracle, golden):
    """With L <= the number of DFT beams the subspace is all of C^L, so the
    learned-subspace solve must reproduce the exact minimum variance."""
    g, s, pr, med, acq = _golden_mv_case(golden)
    cd = O.channel_desc(pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    n0, n1 = len(g["ax0"]), len(g["ax1"])
    cfg = O.bf_config(**dict(BF_CASES["mv"], mv_subarray=4))
    exact = oracle.beamform(cd, g["iq"], g["pts"], n0, n1, cfg, prec="f64")
    v = np.zeros(128, np.float32)
    v[0::2] = 1.0 + 0.5 * np.cos(np.arange(64) * 0.7)
    v[1::2] = 0.3 * np.sin(np.arange(64) * 1.3)
    try:
        oracle.set_lmv_subspace(v, 4, prec="f64")
        sub = oracle.beamform(cd, g["iq"], g["pts"], n0, n1, cfg, prec="f64")
        oracle.set_lmv_subspace(v, 0, prec="f64")
        narrow = oracle.beamform(cd, g["iq"], g["pts"], n0, n1, cfg, prec="f64")
    finally:
        oracle.set_lmv_subspace(None, -1, prec="f64")
    assert rel_l2(sub, exact) < 1e-9
    assert rel_l2(narrow, exact) > 1e-4   # two directions do not span C^4


# ------------------------------------------------------------------ GPU

@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module")
def capi():
    from usx import capi
    return capi


@pytest.fixture(scope="module")
def ctx(capi, torch):
    c = capi.Context(0, stream=0)
    yield c
    c.close()


def _net_case(capi, ctx, torch, rows=384, seed=5):
    rng = np.random.default_rng(seed)
    mlp = capi.Mlp(ctx, DIMS, seed=11)
    p = mlp.get_params()
    # Non-zero biases so that their gradients and the bias epilogue are exercised.
    for w, b in mlp.layers(p):
        b[:] = rng.standard_normal(b.size).astype(np.float32) * 0.1
    mlp.set_params(p)
    x = rng.standard_normal((rows, DIMS[0])).astype(np.float32)
    t = rng.standard_normal((rows, DIMS[-1])).astype(np.float32)
    m = (rng.random((rows, DIMS[-1])) > 0.25).astype(np.float32)
    return mlp, p, x, t, m


@pytest.mark.gpu
def test_mlp_forward_matches_oracle(capi, ctx, torch):
    mlp, p, x, _, _ = _net_case(capi, ctx, torch, rows=300)  # not a multiple of 128: padded internally
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty((x.shape[0], DIMS[-1]), dtype=torch.float32, device="cuda")
    mlp.forward(dx.data_ptr(), x.shape[0], dy.data_ptr())
    ctx.synchronize()
    want, _ = MO.forward(p, DIMS, x, quantize=True)
    assert rel_l2(dy.cpu().numpy(), want) < 2e-3


@pytest.mark.gpu
@pytest.mark.parametrize("dims,rows", [((256, 256), 128), ((256, 128), 384), ((128, 256), 152 * 128 * 3 + 256),
                                       ((256, 384, 128), 1024), ((256, 256, 256, 256, 128), 4096)])
def test_tcgen05_gemm_matches_mma_sync(capi, ctx, torch, dims, rows):
    """The tcgen05 forward GEMM (accumulator in tensor memory) against the
    mma.sync GEMM: the same BF16 products summed in FP32 in another order.
    One layer: within FP32 rounding of a 256-term sum. Several layers: the
    hidden activations are rounded to BF16, so a few outputs may differ by one
    BF16 step of an input. (256, 384, 128) mixes the two paths (a 384-wide
    layer stays on mma.sync); 152 * 128 * 3 + 256 rows give every CTA of the
    persistent grid several tiles."""
    rng = np.random.default_rng(len(dims) * 7 + rows)
    mlp = capi.Mlp(ctx, dims, seed=3)
    p = mlp.get_params()
    for w, b in mlp.layers(p):
        b[:] = rng.standard_normal(b.size).astype(np.float32) * 0.1
    mlp.set_params(p)
    x = rng.standard_normal((rows, dims[0])).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    out = []
    for path in (capi.Mlp.GEMM_AUTO, capi.Mlp.GEMM_MMA_SYNC):
        mlp.set_gemm_path(path)
        dy = torch.full((rows, dims[-1]), float("nan"), dtype=torch.float32, device="cuda")
        mlp.forward(dx.data_ptr(), rows, dy.data_ptr())
        ctx.synchronize()
        out.append(dy.cpu().numpy())
    tc5, mma = out
    assert np.isfinite(tc5).all()
    if len(dims) == 2:
        assert np.abs(tc5 - mma).max() <= 1e-5 * np.abs(mma).max()
        want, _ = MO.forward(p, dims, x, quantize=True)
        assert rel_l2(tc5, want) < 1e-5
    else:
        assert rel_l2(tc5, mma) < 2e-3
        want, _ = MO.forward(p, dims, x, quantize=True)
        assert rel_l2(tc5, want) < 2e-3


@pytest.mark.gpu
def test_mlp_gradients_match_oracle(capi, ctx, torch):
    """Hand-written backward GEMMs (dW split-K, dX with the ReLU mask) and the
    bias reduction against the oracle's backward with the same BF16 rounding."""
    mlp, p, x, t, m = _net_case(capi, ctx, torch)
    dx, dt, dm = (torch.from_numpy(a).cuda() for a in (x, t, m))
    loss, grad = mlp.train_step(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), x.shape[0], 0.0, True, True)
    want_loss, want = MO.backward(p, DIMS, x, t, m, quantize=True)
    assert abs(loss - want_loss) < 1e-3 * want_loss
    o = 0
    for din, dout in zip(DIMS[:-1], DIMS[1:]):
        gw, ww = grad[o:o + din * dout], want[o:o + din * dout]
        o += din * dout
        gb, wb = grad[o:o + dout], want[o:o + dout]
        o += dout
        assert rel_l2(gw, ww) < 3e-3
        assert rel_l2(gb, wb) < 3e-3
    # Parameters are untouched when lr = 0.
    assert np.array_equal(mlp.get_params(), p)


@pytest.mark.gpu
def test_output_loss_gradients_match_oracle(capi, ctx, torch):
    """The learned-MV output loss kernel and the backward through it."""
    mlp, p, x, t, m = _net_case(capi, ctx, torch)
    L = np.random.default_rng(4).integers(2, 65, x.shape[0])
    m = (np.arange(128)[None, :] // 2 < L[:, None]).astype(np.float32)
    t = t + np.tile([4.0, 0.0], 64).astype(np.float32)   # sum(t) away from zero
    mlp.set_loss(capi.Mlp.LOSS_LMV_OUTPUT, 0.05)
    dx, dt, dm = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, t, m))
    loss, grad = mlp.train_step(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), x.shape[0], 0.0, True, True)
    y, _ = MO.forward(p, DIMS, x, quantize=True)
    want_loss, g_out = MO.lmv_output_loss(y, t, m, x, 0.05)
    want = MO.backward_from(p, DIMS, x, g_out, quantize=True)
    assert abs(loss - want_loss) < 2e-3 * want_loss
    assert rel_l2(grad, want) < 5e-3


@pytest.mark.gpu
def test_subspace_loss_gradients_match_oracle(capi, ctx, torch):
    """The learned-subspace direction loss kernel and the backward through it."""
    mlp, p, x, t, m = _net_case(capi, ctx, torch)
    L = np.random.default_rng(6).integers(2, 65, x.shape[0])
    m = (np.arange(128)[None, :] // 2 < L[:, None]).astype(np.float32)
    mlp.set_loss(capi.Mlp.LOSS_LMV_SUBSPACE, 0.05)
    dx, dt, dm = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in (x, t, m))
    loss, grad = mlp.train_step(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), x.shape[0], 0.0, True, True)
    y, _ = MO.forward(p, DIMS, x, quantize=True)
    want_loss, g_out = MO.lmv_subspace_loss(y, t, m, 0.05)
    want = MO.backward_from(p, DIMS, x, g_out, quantize=True)
    assert abs(loss - want_loss) < 2e-3 * want_loss
    assert rel_l2(grad, want) < 5e-3


@pytest.mark.gpu
def test_adam_step_matches_oracle(capi, ctx, torch):
    mlp, p, x, t, m = _net_case(capi, ctx, torch)
    dx, dt, dm = (torch.from_numpy(a).cuda() for a in (x, t, m))
    _, g = mlp.train_step(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), x.shape[0], 0.0, False, True)
    lr = 1e-3
    mlp.train_step(dx.data_ptr(), dt.data_ptr(), dm.data_ptr(), x.shape[0], lr)
    got = mlp.get_params()
    want, _, _ = MO.adam_step(p.astype(np.float64), g.astype(np.float64), 0.0, 0.0, 1, lr)
    step = got - p
    # The first Adam step moves each parameter by ~lr * sign(g); split-K
    # accumulation order may flip only the tiniest gradients.
    assert rel_l2(step, want - p) < 1e-2
    assert np.mean(np.abs(step - (want - p)) > 1e-5) < 1e-3


@pytest.mark.gpu
def test_training_drives_the_loss_down(capi, ctx, torch):
    """A smooth target (a fixed random network) is learned by the on-device loop."""
    rng = np.random.default_rng(1)
    rows = 4096
    x = rng.standard_normal((rows, DIMS[0])).astype(np.float32)
    teacher = capi.Mlp(ctx, DIMS, seed=99)
    dx = torch.from_numpy(x).cuda()
    dt = torch.empty((rows, DIMS[-1]), dtype=torch.float32, device="cuda")
    teacher.forward(dx.data_ptr(), rows, dt.data_ptr())
    student = capi.Mlp(ctx, DIMS, seed=3)
    first = None
    for step in range(300):
        loss, _ = student.train_step(dx.data_ptr(), dt.data_ptr(), None, rows, 1e-3, step % 50 == 0 or step == 299)
        if loss is not None:
            first = loss if first is None else first
            last = loss
    assert last < 0.5 * first


def _learned_setup():
    from usx import learned
    return learned, learned.Setup(n_tx=15, depth=0.04, n0=128, n1=256)


@pytest.mark.gpu
def test_features_and_weights_match_oracle(capi, torch, oracle):
    """Device features (trapezoid-weighted lag products) and tensor-core Capon
    weights against the oracle's direct definitions, on a simulated phantom."""
    learned, setup = _learned_setup()
    im = learned.Imager(setup)
    try:
        spec = learned.phantom(7, setup)
        im.acquire(spec)
        frame, feat, w, valid = im.export_pairs()
        iq = im.iq.cpu().numpy()
        feat, w, valid = feat.cpu().numpy(), w.cpu().numpy(), valid.cpu().numpy()
        # The oracle on a band of 8 lateral lines (the oracle is a plain CPU loop).
        lines = np.arange(60, 68)
        pts = im.grid.points.reshape(setup.n0, setup.n1, 3)[lines].reshape(-1, 3)
        pr = O.probe(n_elements=setup.n_el, pitch=setup.pitch, element_width=setup.width,
                     center_frequency=setup.f0, bandwidth=0.6)
        a = im.ch_iq.desc.acq
        acq = O.acquisition(fs=a.sampling_frequency, n_samples=a.n_samples, t0=a.t0, prf=a.prf)
        tx = im.transmits
        n = len(tx)
        txs = O.TxSet(np.array([t["type"] for t in tx]), np.array([t["angle"] for t in tx], np.float32),
                      np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32),
                      np.stack([np.asarray(t["delays"], np.float32) for t in tx]),
                      np.stack([np.asarray(t["apodization"], np.float32) for t in tx]))
        cd = O.channel_desc(pr, O.medium(), acq, txs, is_iq=True, fdem=setup.f0)
        fr_o, feat_o, w_o, valid_o = oracle.mv_training_pairs(cd, iq, pts, len(lines), setup.n1,
                                                              O.bf_config(**setup_bf_kw(setup)))
        rows = (lines[:, None] * setup.n1 + np.arange(setup.n1)[None, :]).ravel()
        assert np.array_equal(valid[rows], valid_o)
        ok = valid_o == 1
        assert np.max(np.abs(feat[rows] - feat_o)) < 2e-3
        # Weights: the tensor-core solve is within 1e-3 of the exact frame;
        # normalised weights of well-conditioned pixels agree to ~1e-2.
        wc, wo = w[rows][ok], w_o[ok]
        err = np.linalg.norm(wc - wo, axis=1) / np.maximum(np.linalg.norm(wo, axis=1), 1e-12)
        assert np.median(err) < 1e-2
        assert rel_l2(frame.cpu().numpy()[lines], fr_o) < 1e-3
    finally:
        im.close()


def setup_bf_kw(setup):
    return dict(f_number=setup.f_number, combiner=2, mv_subarray=setup.subarray,
                mv_diagonal_loading=setup.loading, mv_range_average=setup.range_avg)


def _uniform_params(mlp):
    """All-zero weights, last bias = (1, 0) per output pair: the network that
    predicts uniform weights w = 1/L (the combiner without learning)."""
    p = np.zeros(mlp.n_params, np.float32)
    _, b = mlp.layers(p)[-1]
    b[0::2] = 1.0
    return p


@pytest.mark.gpu
def test_gate_zero_falls_back_to_plain_mv_everywhere(capi, torch):
    learned, setup = _learned_setup()
    im = learned.Imager(setup)
    try:
        im.acquire(learned.phantom(21, setup))
        mv = im.beamform(learned.COMB_MV).cpu().numpy()
        mlp = capi.Mlp(im.ctx, DIMS, seed=1)
        plan = im.plan(learned.COMB_LEARNED_MV)
        plan.set_learned(mlp, 0.0)
        plan.learned_stats()
        out = im.beamform(learned.COMB_LEARNED_MV).cpu().numpy()
        gated, pixels = plan.learned_stats()
        assert pixels == setup.n0 * setup.n1
        assert gated > 0.9 * pixels
        assert rel_l2(out, mv) < 1e-6
        # With the plan in the FP32 mode its gated pixels take the FP32
        # solver: gate 0 gives that solver's frame.
        mv32_plan = im.ctx.plan(im.ch_iq, im.grid, setup.bf(learned.COMB_MV))
        mv32_plan.set_mv_mode(3)
        mv32 = torch.empty((setup.n0, setup.n1), dtype=torch.complex64, device="cuda")
        mv32_plan.execute(im.iq.data_ptr(), mv32.data_ptr())
        plan.set_mv_mode(3)
        out32 = im.beamform(learned.COMB_LEARNED_MV).cpu().numpy()
        plan.set_mv_mode(0)
        plan.learned_stats()
        mv32_plan.close()
        assert rel_l2(out32, mv32.cpu().numpy()) < 1e-6
        assert rel_l2(out32, mv) < 1e-3
        # An infinite gate takes every network output (no fallback).
        plan.set_learned(mlp, float("inf"))
        im.beamform(learned.COMB_LEARNED_MV)
        gated, pixels = plan.learned_stats()
        assert gated == 0 and pixels == setup.n0 * setup.n1
    finally:
        im.close()


def _constant_net(capi, ctx, v):
    """A network whose output is the vector v for every pixel (zero weights,
    last bias v)."""
    mlp = capi.Mlp(ctx, DIMS, seed=0)
    p = np.zeros(mlp.n_params, np.float32)
    _, b = mlp.layers(p)[-1]
    b[:] = v
    mlp.set_params(p)
    return mlp


@pytest.mark.gpu
@pytest.mark.parametrize("beams", [0, 2, 4, 6])
def test_subspace_refinement_matches_oracle(capi, torch, oracle, beams):
    """The learned-subspace refinement (Capon solve within span{DFT beams,
    network direction}, through the snapshots) against the oracle's
    restatement, which forms the covariance and projects it."""
    learned, setup = _learned_setup()
    im = learned.Imager(setup)
    try:
        im.acquire(learned.phantom(31, setup))
        v = np.zeros(128, np.float32)
        i = np.arange(64)
        v[0::2] = 1.0 + 0.4 * np.cos(2 * np.pi * 3.3 * i / 40.0)
        v[1::2] = 0.25 * np.sin(2 * np.pi * 1.7 * i / 40.0)
        mlp = _constant_net(capi, im.ctx, v)
        plan = im.plan(learned.COMB_LEARNED_MV)
        plan.set_learned(mlp, float("inf"))
        plan.set_learned_refine(beams)
        plan.learned_stats()
        out = im.beamform(learned.COMB_LEARNED_MV).cpu().numpy()
        gated, pixels = plan.learned_stats()
        assert gated == 0
        iq = im.iq.cpu().numpy()
        lines = np.arange(40, 46)
        pts = im.grid.points.reshape(setup.n0, setup.n1, 3)[lines].reshape(-1, 3)
        pr = O.probe(n_elements=setup.n_el, pitch=setup.pitch, element_width=setup.width,
                     center_frequency=setup.f0, bandwidth=0.6)
        a = im.ch_iq.desc.acq
        acq = O.acquisition(fs=a.sampling_frequency, n_samples=a.n_samples, t0=a.t0, prf=a.prf)
        tx = im.transmits
        n = len(tx)
        txs = O.TxSet(np.array([t["type"] for t in tx]), np.array([t["angle"] for t in tx], np.float32),
                      np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32),
                      np.stack([np.asarray(t["delays"], np.float32) for t in tx]),
                      np.stack([np.asarray(t["apodization"], np.float32) for t in tx]))
        cd = O.channel_desc(pr, O.medium(), acq, txs, is_iq=True, fdem=setup.f0)
        # The oracle in float (its channel samples are the reference's to the
        # bit); the minimum-variance family amplifies FP32 rounding to ~1e-3
        # against an FP64 evaluation, so the FP32 oracle is the like-for-like check.
        try:
            oracle.set_lmv_subspace(v, beams, prec="f32")
            want = oracle.beamform(cd, iq, pts, len(lines), setup.n1, O.bf_config(**setup_bf_kw(setup)))
        finally:
            oracle.set_lmv_subspace(None, -1, prec="f32")
        got = out[lines]
        mv = oracle.beamform(cd, iq, pts, len(lines), setup.n1, O.bf_config(**setup_bf_kw(setup)))
        err, err_mv = rel_l2(got, want), rel_l2(got, mv)
        assert err < 1e-3
        # The refinement is a proper approximation of plain MV here, not MV itself.
        assert rel_l2(want, mv) > 3e-3 and err < 0.2 * err_mv
    finally:
        im.close()


@pytest.mark.gpu
def test_learned_plan_needs_a_network(capi, torch):
    learned, setup = _learned_setup()
    im = learned.Imager(setup)
    try:
        im.acquire(learned.phantom(22, setup))
        with pytest.raises(ValueError, match="no network"):
            im.beamform(learned.COMB_LEARNED_MV)
        wrong = capi.Mlp(im.ctx, (128, 128), seed=0)
        with pytest.raises(ValueError, match="256 features"):
            im.plan(learned.COMB_LEARNED_MV).set_learned(wrong, 0.05)
    finally:
        im.close()


@pytest.mark.gpu
def test_training_gains_over_uniform_weights(capi, torch):
    """Trained on plain-MV pairs from 12 phantoms, the network's images are
    closer to plain MV (relative L2, wire lateral FWHM) on held-out phantoms
    than the same combiner with uniform weights (the method without it)."""
    learned, setup = _learned_setup()
    im = learned.Imager(setup)
    try:
        X, T, M = learned.make_pairs(im, np.arange(100, 112), per_phantom=8192, log=None)
        mlp, losses = learned.train(im.ctx, X, T, M, steps=1500, batch=2048, lr=1e-3, log=None)
        assert losses[-1][1] < losses[0][1]
        uniform = capi.Mlp(im.ctx, DIMS)
        uniform.set_params(_uniform_params(uniform))
        plan = im.plan(learned.COMB_LEARNED_MV)
        res = {}
        for name, net in (("trained", mlp), ("uniform", uniform)):
            plan.set_learned(net, float("inf"))
            errs, fw = [], []
            for s in (900, 901):
                spec = learned.phantom(s, setup)
                im.acquire(spec)
                mv = im.beamform(learned.COMB_MV)
                lf = im.beamform(learned.COMB_LEARNED_MV)
                errs.append(float((lf - mv).abs().pow(2).sum().sqrt() / mv.abs().pow(2).sum().sqrt()))
                a, b = learned.image_metrics(mv, im, spec), learned.image_metrics(lf, im, spec)
                fw += [abs(y - x) / x for x, y in zip(a["lateral_fwhm_mm"], b["lateral_fwhm_mm"])]
            res[name] = (np.mean(errs), np.mean(fw))
        assert res["trained"][0] < 0.8 * res["uniform"][0], res
        assert res["trained"][1] < res["uniform"][1], res
    finally:
        im.close()


@pytest.mark.gpu
def test_shipped_network_gains_over_the_beams_alone(capi, torch):
    """The shipped configuration (the shipped network, the subspace refinement
    with its recorded beams, 128 channels, 75 plane waves, 512 x 1024) against
    the same refinement without the network's direction, on two held-out
    phantoms: with the network the frame is closer to plain minimum variance
    (relative L2), i.e. the trained network is what the method gains over the
    DFT beams alone."""
    from usx import learned
    if not learned.DEFAULT_WEIGHTS.exists():
        pytest.fail("the shipped network weights are missing")
    im = learned.Imager(learned.Setup())
    try:
        mlp = learned.load_mlp(im.ctx)
        plan = im.plan(learned.COMB_LEARNED_MV)
        plan.set_learned(mlp, float("inf"))
        plan.set_learned_refine(max(0, learned.trained_refine()))
        err = {True: [], False: []}
        for seed in (900_000, 900_001):
            im.acquire(learned.phantom(seed, im.setup), noise_seed=seed)
            mv = im.beamform(learned.COMB_MV)
            for use_net in (True, False):
                plan.set_learned_subspace(use_net, float("inf"))
                lf = im.beamform(learned.COMB_LEARNED_MV)
                err[use_net].append(float((lf - mv).abs().pow(2).sum().sqrt() / mv.abs().pow(2).sum().sqrt()))
        assert np.mean(err[True]) < 0.9 * np.mean(err[False]), err
        mlp.close()
    finally:
        im.close()


@pytest.mark.gpu
def test_share_gate_sends_pixels_to_the_exact_solver(capi, torch):
    """The gate on the network direction's share of the power reduction: at 0
    every pixel whose refinement used the network goes to the exact solver,
    and the frame is then plain minimum variance wherever it did; at +inf no
    pixel is gated by it; in between the fallback rate falls as the gate rises."""
    from usx import learned
    im = learned.Imager(learned.Setup(n_tx=15, depth=0.04, n0=128, n1=256))
    try:
        mlp = learned.load_mlp(im.ctx)
        plan = im.plan(learned.COMB_LEARNED_MV)
        plan.set_learned(mlp, float("inf"))
        plan.set_learned_refine(6)
        im.acquire(learned.phantom(31, im.setup))
        mv = im.beamform(learned.COMB_MV)
        rates = []
        for share in (0.0, 0.05, 0.3, float("inf")):
            plan.set_learned_subspace(True, share)
            plan.learned_stats()
            lf = im.beamform(learned.COMB_LEARNED_MV)
            gated, pixels = plan.learned_stats()
            rates.append(gated / max(1, pixels))
            if share == 0.0:
                err0 = float((lf - mv).abs().pow(2).sum().sqrt() / mv.abs().pow(2).sum().sqrt())
        assert rates[0] > 0.5 and rates[-1] < 1e-3, rates
        assert rates[0] >= rates[1] >= rates[2] >= rates[3], rates
        assert err0 < 2e-3, err0
        with pytest.raises(ValueError):
            plan.set_learned_subspace(True, -1.0)
        mlp.close()
    finally:
        im.close()


@pytest.mark.gpu
def test_level_gate_sends_bright_pixels_to_the_exact_solver(capi, torch):
    """The gate on tr(R) over its depth's level (the geometric mean over the
    lateral lines): at ratio 1 roughly every pixel brighter than its depth's
    level goes to the exact solver, at +inf none, and the rate falls as the
    ratio rises; the pixels around a bright wire are among the first gated."""
    from usx import learned
    im = learned.Imager(learned.Setup(n_tx=15, depth=0.04, n0=128, n1=256))
    try:
        mlp = learned.load_mlp(im.ctx)
        plan = im.plan(learned.COMB_LEARNED_MV)
        plan.set_learned(mlp, float("inf"))
        plan.set_learned_refine(6)
        spec = learned.phantom(31, im.setup)
        im.acquire(spec)
        im.beamform(learned.COMB_MV)
        rates = []
        for level in (1.0, 3.0, 30.0, float("inf")):
            plan.set_learned_level_gate(level)
            plan.learned_stats()
            im.beamform(learned.COMB_LEARNED_MV)
            gated, pixels = plan.learned_stats()
            rates.append(gated / max(1, pixels))
        assert 0.2 < rates[0] < 0.9 and rates[-1] < 1e-3, rates
        assert rates[0] >= rates[1] >= rates[2] >= rates[3], rates
        # A neighbourhood gates the flanks with the hot pixels: more pixels
        # at the same ratio, growing with the window.
        wrates = []
        plan.set_learned_level_gate(3.0)
        for win in ((0, 0), (1, 2), (3, 6)):
            plan.set_learned_level_window(*win)
            plan.learned_stats()
            im.beamform(learned.COMB_LEARNED_MV)
            gated, pixels = plan.learned_stats()
            wrates.append(gated / max(1, pixels))
        assert wrates[0] == pytest.approx(rates[1]) and wrates[0] < wrates[1] < wrates[2] < 1.0, wrates
        with pytest.raises(ValueError):
            plan.set_learned_level_window(-1, 0)
        plan.set_learned_level_window(0, 0)
        with pytest.raises(ValueError):
            plan.set_learned_level_gate(0.5)
        mlp.close()
    finally:
        im.close()
