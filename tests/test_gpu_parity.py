"""CUDA kernels against the reference (golden fixtures) and the CPU oracle,
called through the C-ABI (libusx_cu.so via usx.capi), device memory from torch.

Tolerances (relative L2 unless stated):
  FP32 paths (demodulation, DAS/CF/DMAS in every compounding mode, RF
  beamforming, the simulator, envelope, TGC, log compression, scan conversion,
  wall filter, power Doppler, displacement, strain):           <= 1e-5
  minimum variance (FP32 covariance and Cholesky in the reference's order;
  a Cholesky solve amplifies rounding by the condition number): <= 1e-4
  colour-flow velocity: equal validity masks except at most 1% of pixels at
  a gate boundary, velocities where both valid within 1e-4 relative.
The kernels follow the reference's operation order without FMA contraction,
so most of these agree to the last ulp of the device's sincosf/cosf/atan2f.
"""

from __future__ import annotations

import numpy as np
import pytest

from gold import BF_CASES, rel_l2, sim_setup, txset
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_MV = 1e-4


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


@pytest.fixture(scope="module")
def capi():
    from usx import capi as c
    return c


@pytest.fixture(scope="module")
def ctx(capi, torch):
    c = capi.Context(0, stream=torch.cuda.current_stream().cuda_stream)
    yield c
    c.close()


def dev(torch, a):
    a = np.ascontiguousarray(a)
    return torch.from_numpy(a).cuda()


def host(torch, t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def c_probe(capi, p):
    return capi.Probe(p.n_elements, p.pitch, p.element_width, p.elevation_height, p.center_frequency, p.bandwidth)


def c_channel(capi, pr, med, acq, txs: O.TxSet, is_iq=False, fdem=0.0):
    tx = [dict(type=int(txs.types[e]), angle=float(txs.angles[e]), focus=txs.focus[e], origin=txs.origin[e],
               delays=txs.delays[e], apodization=txs.apod[e]) for e in range(len(txs))]
    return capi.Channel(c_probe(capi, pr), capi.Medium(med.speed_of_sound, med.attenuation, med.density),
                        capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf), tx, is_iq, fdem)


# --------------------------------------------------------------- simulator

def test_simulate_matches_reference(capi, ctx, torch, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    ch = c_channel(capi, pr, med, acq, txset(g, "pw"))
    scat = dev(torch, g["scat"])
    z = dev(torch, g["noise_z"])
    rf = torch.empty(g["rf"].shape, dtype=torch.float32, device="cuda")
    stats = ctx.simulate(ch, capi.sim_config(noise_db=-60.0, noise_seed=7), scat.data_ptr(), len(g["scat"]),
                         z.data_ptr(), rf.data_ptr(), want_stats=True)
    assert rel_l2(host(torch, rf), g["rf"]) < TOL
    assert stats[0] > 0
    ctx.simulate(ch, capi.sim_config(noise_db=-200.0, incident_trim_db=-30.0, enable_motion=0), scat.data_ptr(),
                 len(g["scat"]), None, rf.data_ptr())
    assert rel_l2(host(torch, rf), g["rf_quiet"]) < TOL


def test_simulate_focused_and_no_diffraction_match_oracle(capi, ctx, torch, golden, oracle):
    g = golden("sim")
    b = golden("bf")
    pr, med, acq = sim_setup(g)
    for txs, cfg in ((txset(b, "foc"), dict(noise_db=-200.0)),
                     (txset(g, "pw"), dict(noise_db=-200.0, full_transmit_diffraction=0, apply_attenuation=0)),
                     (txset(b, "div"), dict(noise_db=-200.0, apply_directivity=0, oversampling=2))):
        ch = c_channel(capi, pr, med, acq, txs)
        rf = torch.empty((len(txs), pr.n_elements, acq.n_samples), dtype=torch.float32, device="cuda")
        sc = dev(torch, g["scat"])
        ctx.simulate(ch, capi.sim_config(**cfg), sc.data_ptr(), len(g["scat"]), None, rf.data_ptr())
        want = oracle.simulate(O.channel_desc(pr, med, acq, txs), O.sim_config(**cfg), g["scat"])
        assert rel_l2(host(torch, rf), want) < TOL


def test_simulate_is_deterministic(capi, ctx, torch, golden):
    """No floating-point atomics: every RF sample sums its scatterers in the
    same order, so two runs (and a run with the scatterers' memory reused)
    give bit-identical RF, noise included."""
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    ch = c_channel(capi, pr, med, acq, txset(g, "pw"))
    scat = dev(torch, np.concatenate([g["scat"]] * 20))  # 12,840 scatterers, many per RF sample
    z = dev(torch, g["noise_z"])
    out = []
    for _ in range(2):
        rf = torch.full(g["rf"].shape, float("nan"), dtype=torch.float32, device="cuda")
        ctx.simulate(ch, capi.sim_config(noise_db=-60.0, noise_seed=7), scat.data_ptr(), scat.shape[0],
                     z.data_ptr(), rf.data_ptr())
        out.append(host(torch, rf))
    assert np.isfinite(out[0]).all()
    assert np.array_equal(out[0], out[1])


def test_simulate_empty_phantom_and_zero_amplitudes(capi, ctx, torch, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    ch = c_channel(capi, pr, med, acq, txset(g, "pw"))
    rf = torch.full(g["rf"].shape, 7.0, dtype=torch.float32, device="cuda")
    ctx.simulate(ch, capi.sim_config(noise_db=-200.0), 0, 0, None, rf.data_ptr())
    assert float(host(torch, rf).__abs__().max()) == 0.0
    scat = g["scat"].copy()
    scat[:, 3] = 0.0
    sc, z = dev(torch, scat), dev(torch, g["noise_z"])
    ctx.simulate(ch, capi.sim_config(noise_db=-60.0), sc.data_ptr(), len(scat), z.data_ptr(), rf.data_ptr())
    assert float(np.abs(host(torch, rf)).max()) == 0.0  # zero peak: no noise either


# ------------------------------------------------------------- demodulator

@pytest.mark.parametrize("key,kw", [("iq", {}), ("iq_dec2", dict(decimation=2, filter_taps=21, cutoff_fraction=0.45))])
def test_demodulate_matches_reference(capi, ctx, torch, golden, key, kw):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    ch = c_channel(capi, pr, med, acq, txset(g, "pw"))
    want = g[key]
    iq = torch.empty(want.shape, dtype=torch.complex64, device="cuda")
    rf = dev(torch, g["rf"])
    fdem = ctx.demodulate(ch, capi.demod_config(**kw), rf.data_ptr(), iq.data_ptr())
    assert fdem == pytest.approx(5e6)
    assert rel_l2(host(torch, iq), want) < TOL


def test_demodulate_rejects_iq_input(capi, ctx, torch, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    ch = c_channel(capi, pr, med, acq, txset(g, "pw"), is_iq=True, fdem=5e6)
    buf = torch.empty(16, device="cuda")
    with pytest.raises(ValueError):
        ctx.demodulate(ch, capi.demod_config(), buf.data_ptr(), buf.data_ptr())


# --------------------------------------------------------------- beamformer

def _bf(capi, ctx, torch, ch, grid, cfg, data, ev_begin=0, ev_end=-1):
    plan = ctx.plan(ch, grid, cfg, ev_begin, ev_end)
    out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
    d = dev(torch, data)
    plan.execute(d.data_ptr(), out.data_ptr())
    res = host(torch, out)
    plan.close()
    return res


@pytest.mark.parametrize("name", sorted(BF_CASES))
def test_beamform_matches_reference(capi, ctx, torch, golden, name):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    out = _bf(capi, ctx, torch, ch, grid, capi.bf_config(**BF_CASES[name]), g["iq"])
    tol = TOL_MV if name.startswith("mv") else TOL
    assert rel_l2(out, g[f"bf_{name}"]) < tol


@pytest.mark.parametrize("name", ["das", "cf", "dmas", "incoh", "select", "mv"])
def test_exact_precision_matches_reference_to_the_ulp(capi, ctx, torch, golden, name):
    """USX_BF_EXACT evaluates every operation in the reference's order: only the
    1-ulp differences of the device's sincosf/cosf remain."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    plan = ctx.plan(ch, grid, capi.bf_config(**BF_CASES[name]))
    plan.set_precision(1)
    out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
    d = dev(torch, g["iq"])
    plan.execute(d.data_ptr(), out.data_ptr())
    got = host(torch, out)
    plan.close()
    assert rel_l2(got, g[f"bf_{name}"]) < (1e-5 if name == "mv" else 1e-6)


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("name", ["mv", "mv_l4", "mv_cf"])
def test_mv_tensor_cores_match_reference(capi, ctx, torch, golden, name, mode):
    """BF16 tensor-core covariance (mode 1: batched rank-K update on tcgen05;
    mode 2: warp-level mma.sync) + FP32 refinement: within 1e-3 of the
    reference; mode 3 (FP32 covariance by the lag recurrence, one FP32
    solve, no refinement): within 1e-5, the reference's own precision."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    plan = ctx.plan(ch, grid, capi.bf_config(**BF_CASES[name]))
    plan.set_mv_mode(mode)
    out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
    d = dev(torch, g["iq"])
    plan.execute(d.data_ptr(), out.data_ptr())
    got = host(torch, out)
    fp64, failed = plan.mv_stats()
    plan.close()
    assert rel_l2(got, g[f"bf_{name}"]) < (1e-5 if mode == 3 else 1e-3)
    assert failed == 0
    if mode == 3:
        assert fp64 == 0  # no refinement, so no FP64 re-solve


@pytest.mark.parametrize("mode", [1, 3])
def test_mv_tensor_cores_on_sector_grid(capi, ctx, torch, golden, mode):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    chd = c_channel(capi, pr, med, acq, txset(g, "div"), is_iq=True, fdem=5e6)
    sgrid = capi.Grid(1, g["sax0"], g["sax1"], g["spts"])
    plan = ctx.plan(chd, sgrid, capi.bf_config(f_number=1.5, combiner=2, mv_subarray=12))
    plan.set_mv_mode(mode)
    out = torch.empty(sgrid.shape, dtype=torch.complex64, device="cuda")
    d = dev(torch, g["div_iq"])
    plan.execute(d.data_ptr(), out.data_ptr())
    assert rel_l2(host(torch, out), g["bf_div_mv"]) < (1e-5 if mode == 3 else 1e-3)
    plan.close()


def test_beamform_geometries_match_reference(capi, ctx, torch, golden):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    assert rel_l2(_bf(capi, ctx, torch, ch, grid, capi.bf_config(f_number=1.5), g["iq"], 1, 2), g["bf_das_ev1"]) < TOL
    chr_ = c_channel(capi, pr, med, acq, txset(s, "pw"))
    assert rel_l2(_bf(capi, ctx, torch, chr_, grid, capi.bf_config(f_number=1.5), s["rf"]), g["bf_rf"]) < TOL
    chf = c_channel(capi, pr, med, acq, txset(g, "foc"), is_iq=True, fdem=5e6)
    assert rel_l2(_bf(capi, ctx, torch, chf, grid, capi.bf_config(f_number=1.5, compounding=2), g["foc_iq"]),
                  g["bf_foc_select"]) < TOL
    assert rel_l2(_bf(capi, ctx, torch, chf, grid, capi.bf_config(f_number=1.5), g["foc_iq"]), g["bf_foc_coh"]) < TOL
    chd = c_channel(capi, pr, med, acq, txset(g, "div"), is_iq=True, fdem=5e6)
    sgrid = capi.Grid(1, g["sax0"], g["sax1"], g["spts"])
    assert rel_l2(_bf(capi, ctx, torch, chd, sgrid, capi.bf_config(f_number=1.5), g["div_iq"]), g["bf_div_sector"]) < TOL
    assert rel_l2(_bf(capi, ctx, torch, chd, sgrid, capi.bf_config(f_number=1.5, combiner=2, mv_subarray=12),
                      g["div_iq"]), g["bf_div_mv"]) < TOL_MV


@pytest.mark.parametrize("cfg_kw", [dict(f_number=1.5), dict(f_number=1.5, combiner=1),
                                    dict(f_number=1.5, coherence_factor=1), dict(f_number=1.5, compounding=2)])
def test_das_variants_bit_identical_and_autotune(capi, ctx, torch, golden, cfg_kw):
    """Every delay-and-sum launch shape gives the same frame bit for bit
    (the channel-warp kernels combine the channels in shared memory in the
    same order); the autotuner keeps one of them and leaves its frame in the
    output."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    plan = ctx.plan(ch, grid, capi.bf_config(**cfg_kw))
    d = dev(torch, g["iq"])
    out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
    frames = []
    variants = capi.das_variants()
    assert len(variants) >= 2 and variants[0] == (8, 4, 8, 1, 0, 0)
    assert any(v[4] == 1 for v in variants)  # deepest-tiles-first orders are candidates
    assert any(v[5] == 2 for v in variants)  # transmit-table kernels are candidates
    assert any(v[5] == 4 for v in variants)  # channel-warp kernels are candidates
    for v in range(len(variants)):
        plan.set_variant(v)
        plan.execute(d.data_ptr(), out.data_ptr())
        frames.append(host(torch, out))
    for f in frames[1:]:
        assert np.array_equal(f, frames[0])
    out.zero_()
    best, ms = plan.autotune(d.data_ptr(), out.data_ptr(), repeats=1)
    assert 0 <= best < len(variants) and plan.variant() == best
    assert len(ms) == len(variants) and all(m > 0 for m in ms) and ms[best] == min(ms)
    assert np.array_equal(host(torch, out), frames[0])
    with pytest.raises(ValueError):
        plan.set_variant(len(variants))
    plan.close()


def test_mv_export_variants_bit_identical(capi, ctx, torch, golden):
    """Minimum variance through every delay-and-sum shape, including the
    channel-warp tabulated kernels: the exported channel samples are the same
    bit for bit, so the FP32 minimum-variance frames are identical; on a ragged
    grid too."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    ax0, ax1 = np.asarray(g["ax0"]), np.asarray(g["ax1"])
    pts = np.asarray(g["pts"], dtype=np.float32).reshape(len(ax0), len(ax1), 3)
    d = dev(torch, g["iq"])
    variants = capi.das_variants()
    assert any(v[5] == 4 for v in variants)  # channel-warp shapes are candidates
    grids = (capi.Grid(0, ax0, ax1, pts.reshape(-1, 3)), capi.Grid(0, ax0[:13], ax1[:37], pts[:13, :37].reshape(-1, 3)))
    for gi, grid in enumerate(grids):
        plan = ctx.plan(ch, grid, capi.bf_config(**BF_CASES["mv"]))
        plan.set_mv_mode(3)
        out = torch.empty(grid.shape, dtype=torch.complex64, device="cuda")
        frames = []
        for v in range(len(variants)):
            plan.set_variant(v)
            out.fill_(float("nan"))
            plan.execute(d.data_ptr(), out.data_ptr())
            frames.append(host(torch, out))
        for v, f in enumerate(frames[1:], 1):
            assert np.array_equal(f, frames[0]), f"variant {v}"
        if gi == 0:  # the ragged grid's edge pixels average other range rows
            assert rel_l2(frames[0], g["bf_mv"]) < 1e-5
        plan.close()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg_kw", [dict(f_number=1.5), dict(f_number=1.5, combiner=1, coherence_factor=1)])
def test_das_variants_ragged_grid(capi, ctx, torch, golden, cfg_kw):
    """A grid whose lines and depths do not fill the CTA tiles (13 x 37, tiles
    of 2-8 lines x 32 depths, warps of 1-8 lines): every launch shape gives
    the same frame, bit for bit the same pixels of the full grid."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    ax0, ax1 = np.asarray(g["ax0"]), np.asarray(g["ax1"])
    pts = np.asarray(g["pts"], dtype=np.float32).reshape(len(ax0), len(ax1), 3)
    full = capi.Grid(0, ax0, ax1, pts.reshape(-1, 3))
    sub = capi.Grid(0, ax0[:13], ax1[:37], pts[:13, :37].reshape(-1, 3))
    cfg = capi.bf_config(**cfg_kw)
    d = dev(torch, g["iq"])
    plan_full = ctx.plan(ch, full, cfg)
    out_full = torch.empty(full.shape, dtype=torch.complex64, device="cuda")
    plan_full.execute(d.data_ptr(), out_full.data_ptr())
    want = host(torch, out_full)[:13, :37]
    plan_full.close()
    plan = ctx.plan(ch, sub, cfg)
    out = torch.empty(sub.shape, dtype=torch.complex64, device="cuda")
    for v in range(len(capi.das_variants())):
        plan.set_variant(v)
        out.fill_(float("nan"))
        plan.execute(d.data_ptr(), out.data_ptr())
        assert np.array_equal(host(torch, out), want), f"variant {v}"
    plan.close()


def test_execute_queue_equals_each_plans_own_execution(capi, ctx, torch, golden):
    """Frames of different plans (probe geometry, grid, transmit set, combiner,
    compounding) in one persistent launch: every frame equals its plan's own
    execution bit for bit, including a 75-plane-wave 128-channel frame beside
    the 32-element golden ones, and more entries than one launch takes (the
    call splits them)."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    sgrid = capi.Grid(1, g["sax0"], g["sax1"], g["spts"])
    ch_pw = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    ch_foc = c_channel(capi, pr, med, acq, txset(g, "foc"), is_iq=True, fdem=5e6)
    ch_div = c_channel(capi, pr, med, acq, txset(g, "div"), is_iq=True, fdem=5e6)
    # A large frame of another probe: 128 channels, 75 plane waves, random IQ, 24 x 1024 pixels.
    big_pr = O.probe()
    big_acq = O.acquisition(fs=20e6, n_samples=2073, prf=5000.0)
    ang = np.deg2rad(np.linspace(-16, 16, 75)).astype(np.float32)
    ex = ((np.arange(128, dtype=np.float32) - np.float32(63.5)) * np.float32(300e-6)).astype(np.float32)
    big_tx = O.TxSet(np.ones(75, np.int32), ang, np.tile([0, 0, 0.03], (75, 1)).astype(np.float32),
                     np.zeros((75, 3), np.float32), (ex[None, :] * np.sin(ang)[:, None] / np.float32(1540.0)),
                     np.ones((75, 128), np.float32))
    ch_big = c_channel(capi, big_pr, med, big_acq, big_tx, is_iq=True, fdem=5e6)
    rng = np.random.default_rng(9)
    big_iq = (rng.standard_normal((75, 128, 2073), dtype=np.float32)
              + 1j * rng.standard_normal((75, 128, 2073), dtype=np.float32)).astype(np.complex64)
    bax0 = np.linspace(-0.01, 0.01, 24).astype(np.float32)
    bax1 = np.linspace(0.005, 0.060, 1024).astype(np.float32)
    bpts = np.stack(np.meshgrid(bax0, [0.0], bax1, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    big_grid = capi.Grid(0, bax0, bax1, bpts)
    d_iq, d_foc, d_div, d_big = dev(torch, g["iq"]), dev(torch, g["foc_iq"]), dev(torch, g["div_iq"]), dev(torch, big_iq)
    entries = [(ch_pw, grid, dict(f_number=1.5), d_iq), (ch_pw, grid, dict(f_number=1.5, coherence_factor=1), d_iq),
               (ch_pw, grid, dict(f_number=1.5, combiner=1), d_iq),
               (ch_foc, grid, dict(f_number=1.5, compounding=2), d_foc),
               (ch_div, sgrid, dict(f_number=1.5), d_div), (ch_big, big_grid, dict(f_number=1.5), d_big)]
    plans = [ctx.plan(ch, gr, capi.bf_config(**kw)) for ch, gr, kw, _ in entries]
    want = []
    for p, (_, gr, _, d) in zip(plans, entries):
        out = torch.empty(gr.shape, dtype=torch.complex64, device="cuda")
        p.execute(d.data_ptr(), out.data_ptr())
        want.append(host(torch, out))
    order = list(range(len(plans))) * 9          # 54 entries: two launches
    outs = [torch.full(entries[i][1].shape, float("nan"), dtype=torch.complex64, device="cuda") for i in order]
    ctx.execute_queue([plans[i] for i in order], [entries[i][3].data_ptr() for i in order],
                      [o.data_ptr() for o in outs])
    for i, o in zip(order, outs):
        assert np.array_equal(host(torch, o), want[i]), i
    mv = ctx.plan(ch_pw, grid, capi.bf_config(f_number=1.5, combiner=2))
    with pytest.raises(RuntimeError, match="DAS, DMAS and coherence-factor"):
        ctx.execute_queue([mv], [d_iq.data_ptr()], [outs[0].data_ptr()])
    ch_rf = c_channel(capi, pr, med, acq, txset(s, "pw"))
    rf_plan = ctx.plan(ch_rf, grid, capi.bf_config(f_number=1.5))
    with pytest.raises(ValueError, match="mixed IQ and RF"):
        ctx.execute_queue([plans[0], rf_plan], [d_iq.data_ptr(), d_iq.data_ptr()],
                          [outs[0].data_ptr(), outs[1].data_ptr()])
    for p in plans + [mv, rf_plan]:
        p.close()


def test_batch_and_sequence_equal_single_frames(capi, ctx, torch, golden):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    for cfg in (capi.bf_config(f_number=1.5), capi.bf_config(f_number=1.5, combiner=2, mv_subarray=8)):
        ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
        plan = ctx.plan(ch, grid, cfg)
        iq = g["iq"]
        stack = np.stack([iq, iq * (0.5 + 0.25j), iq[::-1].copy()])
        d = dev(torch, stack)
        n_pix = grid.shape[0] * grid.shape[1]
        out = torch.empty((3, n_pix), dtype=torch.complex64, device="cuda")
        plan.execute_batch(3, d.data_ptr(), iq.size, out.data_ptr(), n_pix)
        got = host(torch, out)
        for f in range(3):
            one = torch.empty(n_pix, dtype=torch.complex64, device="cuda")
            plan.execute(d[f].data_ptr(), one.data_ptr())
            assert np.array_equal(host(torch, one), got[f])
        plan.close()
    # Sequence: each frame beamforms one event; equals beamforming that event alone.
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    plan = ctx.plan(ch, grid, capi.bf_config(f_number=1.5))
    n_pix = grid.shape[0] * grid.shape[1]
    out = torch.empty((3, n_pix), dtype=torch.complex64, device="cuda")
    diq = dev(torch, g["iq"])
    plan.execute_sequence(1, 3, diq.data_ptr(), out.data_ptr(), n_pix)
    got = host(torch, out)
    assert rel_l2(got[1].reshape(grid.shape), g["bf_das_ev1"]) < TOL


def test_beamform_edge_cases(capi, ctx, torch, golden, oracle):
    """Pixels above the face, outside the record and a 4-element probe (n_active
    < 4 falls back to DAS in MV); all against the oracle."""
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    txs = txset(s, "pw")
    n0, n1 = 6, 50
    ax0 = np.linspace(-0.02, 0.02, n0).astype(np.float32)
    ax1 = np.linspace(-0.002, 0.05, n1).astype(np.float32)
    pts = np.stack(np.meshgrid(ax0, [0.0], ax1, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    grid = capi.Grid(0, ax0, ax1, pts)
    for kw in (dict(), dict(combiner=2, mv_subarray=16), dict(combiner=1, coherence_factor=1)):
        ch = c_channel(capi, pr, med, acq, txs, is_iq=True, fdem=5e6)
        got = _bf(capi, ctx, torch, ch, grid, capi.bf_config(**kw), s["iq"])
        want = oracle.beamform(O.channel_desc(pr, med, acq, txs, is_iq=True, fdem=5e6), s["iq"], pts, n0, n1,
                               O.bf_config(**kw))
        assert rel_l2(got, want) < TOL_MV
    small = O.probe(n_elements=4, pitch=300e-6, element_width=270e-6)
    iq4 = np.ascontiguousarray(s["iq"][:, :4, :])
    t4 = O.TxSet(txs.types, txs.angles, txs.focus, txs.origin, txs.delays[:, :4], txs.apod[:, :4])
    ch = c_channel(capi, small, med, acq, t4, is_iq=True, fdem=5e6)
    got = _bf(capi, ctx, torch, ch, grid, capi.bf_config(combiner=2), iq4)
    want = oracle.beamform(O.channel_desc(small, med, acq, t4, is_iq=True, fdem=5e6), iq4, pts, n0, n1,
                           O.bf_config(combiner=2))
    assert rel_l2(got, want) < TOL


def test_beamform_invalid_config_raises(capi, ctx, golden):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    grid = capi.Grid(0, g["ax0"], g["ax1"], g["pts"])
    ch = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    with pytest.raises(ValueError):
        ctx.plan(ch, grid, capi.bf_config(f_number=0.0))
    with pytest.raises(ValueError):
        ctx.plan(ch, grid, capi.bf_config(mv_subarray=1))
    bad = c_channel(capi, pr, med, acq, txset(s, "pw"), is_iq=True, fdem=0.0)
    with pytest.raises(ValueError):
        ctx.plan(bad, grid, capi.bf_config())


# ------------------------------------------------------------ post-process

def test_postprocess_matches_reference(capi, ctx, torch, golden):
    g = golden("post")
    b = golden("bf")
    n0, n1 = g["frame"].shape
    env = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    fr, rfr = dev(torch, g["frame"]), dev(torch, g["rf_frame"])
    ctx.envelope(fr.data_ptr(), n0, n1, 5e6, env.data_ptr())
    assert rel_l2(host(torch, env), g["env_iq"]) < TOL
    ctx.envelope(rfr.data_ptr(), n0, n1, 0.0, env.data_ptr())
    assert rel_l2(host(torch, env), g["env_rf"]) < TOL
    # Inputs are held in named tensors: a temporary's memory would be reused by
    # torch's caching allocator for the next upload while the kernel reads it.
    out = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    env_iq, pts, tgc = dev(torch, g["env_iq"]), dev(torch, b["pts"]), dev(torch, g["tgc"])
    ctx.apply_tgc(env_iq.data_ptr(), n0, n1, pts.data_ptr(), 0.5, 5e6, out.data_ptr())
    assert rel_l2(host(torch, out), g["tgc"]) < TOL
    ctx.log_compress(tgc.data_ptr(), n0 * n1, 50.0, 2.0, -1.0, out.data_ptr())
    assert rel_l2(host(torch, out), g["log"]) < TOL
    ctx.log_compress(tgc.data_ptr(), n0 * n1, 40.0, 0.0, float(g["tgc"].max() * 0.5), out.data_ptr())
    assert rel_l2(host(torch, out), g["log_ref"]) < TOL
    sgrid = capi.Grid(1, b["sax0"], b["sax1"], b["spts"])
    px = torch.empty((40, 50), dtype=torch.float32, device="cuda")
    img = dev(torch, g["sc_img"])
    ext = ctx.scan_convert(img.data_ptr(), sgrid, 50, 40, -1.0, px.data_ptr())
    assert rel_l2(host(torch, px), g["sc_sector"]) < TOL
    assert np.array_equal(ext, g["sc_sector_ext"])
    cgrid = capi.Grid(0, b["ax0"], b["ax1"], b["pts"])
    px = torch.empty((47, 33), dtype=torch.float32, device="cuda")
    ctx.scan_convert(env_iq.data_ptr(), cgrid, 33, 47, 0.0, px.data_ptr())
    assert rel_l2(host(torch, px), g["sc_cart"]) < TOL


def test_scan_convert_tiles_and_extent_match_oracle(capi, ctx, torch, oracle):
    """Rasters of several 32 x 32 tiles with ragged edges (75 x 131, 33 x 64,
    1 x 1), a Cartesian grid (bit-exact: no transcendental on that path) and a
    sector grid (atan2f, 1e-5); and the extent scan's tie rule: with +0.0 and
    -0.0 both minimal depths, the first in point order is returned, as by one
    sequential std::min pass."""
    rng = np.random.default_rng(11)
    n0, n1 = 97, 161  # 15617 points: the extent scan's quarters leave a tail
    ax0 = np.linspace(-0.019, 0.019, n0, dtype=np.float32)
    ax1 = np.linspace(0.0, 0.045, n1, dtype=np.float32)
    pts = np.zeros((n0 * n1, 3), np.float32)
    pts[:, 0] = np.repeat(ax0, n1)
    pts[:, 2] = np.tile(ax1, n0)
    img = rng.random((n0, n1), dtype=np.float32)
    d_img = dev(torch, img)
    for first_sign in (1.0, -1.0):
        p = pts.copy()
        p[::n1, 2] = 0.0
        p[0, 2] = first_sign * 0.0
        p[(n0 - 3) * n1, 2] = -first_sign * 0.0
        cgrid = capi.Grid(0, ax0, ax1, p)
        for w, h in ((75, 131), (33, 64), (1, 1)):
            px = torch.empty((h, w), dtype=torch.float32, device="cuda")
            ext = ctx.scan_convert(d_img.data_ptr(), cgrid, w, h, -2.0, px.data_ptr())
            want, want_ext = oracle.scan_convert(img, 0, ax0, ax1, (0, 0, 0), p, w, h, -2.0)
            assert np.array_equal(host(torch, px), want), (w, h)
            assert np.array_equal(ext, want_ext)
            assert np.signbit(ext[2]) == (first_sign < 0)
    th = np.linspace(-0.6, 0.6, n0, dtype=np.float32)
    r = np.linspace(0.01, 0.08, n1, dtype=np.float32)
    sp = np.zeros((n0 * n1, 3), np.float32)
    sp[:, 0] = (np.sin(th)[:, None] * r[None, :]).ravel()
    sp[:, 2] = (np.cos(th)[:, None] * r[None, :]).ravel()
    sgrid = capi.Grid(1, th, r, sp)
    px = torch.empty((131, 75), dtype=torch.float32, device="cuda")
    ext = ctx.scan_convert(d_img.data_ptr(), sgrid, 75, 131, -1.0, px.data_ptr())
    want, want_ext = oracle.scan_convert(img, 1, th, r, (0, 0, 0), sp, 75, 131, -1.0)
    assert np.array_equal(ext, want_ext)
    assert rel_l2(host(torch, px), want) < TOL


# ---------------------------------------------------------- Doppler / strain

@pytest.mark.parametrize("key,wt,order", [("w0o1", 0, 1), ("w1o1", 1, 1), ("w1o2", 1, 2), ("w2o0", 2, 0)])
def test_doppler_matches_reference(capi, ctx, torch, golden, key, wt, order):
    g = golden("doppler")
    ens = g["ens"]
    n, n0, n1 = ens.shape
    d = dev(torch, ens)
    out = torch.empty_like(d)
    ctx.wall_filter(d.data_ptr(), n, n0 * n1, wt, order, out.data_ptr())
    assert rel_l2(host(torch, out), g[f"wall_{key}"]) < TOL
    pw = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    ctx.power_doppler(d.data_ptr(), n, n0 * n1, wt, order, pw.data_ptr())
    assert rel_l2(host(torch, pw), g[f"pd_{key}"]) < TOL
    vel, pwr, var = (torch.empty((n0, n1), dtype=torch.float32, device="cuda") for _ in range(3))
    valid = torch.empty((n0, n1), dtype=torch.uint8, device="cuda")
    nyq = ctx.color_flow(d.data_ptr(), n, n0, n1, g["ax1"], 5e6, 5000.0, 1540.0,
                         capi.doppler_config(wall_filter=wt, polynomial_order=order),
                         vel.data_ptr(), pwr.data_ptr(), var.data_ptr(), valid.data_ptr())
    assert np.float32(nyq) == g[f"cf_nyq_{key}"]
    v, vd = host(torch, vel), host(torch, valid)
    assert rel_l2(host(torch, pwr), g[f"cf_pow_{key}"]) < TOL
    assert np.mean(vd != g[f"cf_valid_{key}"]) <= 0.01
    both = (vd == 1) & (g[f"cf_valid_{key}"] == 1)
    assert rel_l2(v[both], g[f"cf_vel_{key}"][both]) < 1e-4


def test_color_flow_batch_of_uneven_ensembles(capi, ctx, torch, golden, oracle):
    g = golden("doppler")
    ens = g["ens"]
    n, n0, n1 = ens.shape
    lens = [4, 10, 6, 2]
    frames = np.concatenate([ens[:k] for k in lens])
    offs = np.cumsum([0] + lens[:-1])
    d = dev(torch, frames)
    cfg = capi.doppler_config(wall_filter=1, polynomial_order=1)
    vel, pwr, var = (torch.empty((len(lens), n0, n1), dtype=torch.float32, device="cuda") for _ in range(3))
    valid = torch.empty((len(lens), n0, n1), dtype=torch.uint8, device="cuda")
    ctx.color_flow_batch(d.data_ptr(), lens, offs, n0, n1, g["ax1"], 5e6, 5000.0, 1540.0, cfg, vel.data_ptr(),
                         pwr.data_ptr(), var.data_ptr(), valid.data_ptr())
    P = host(torch, pwr)
    for e, k in enumerate(lens):
        _, p, _, _, _ = oracle.color_flow(ens[:k], g["ax1"], 5e6, 5000.0, 1540.0, O.doppler_config())
        assert rel_l2(P[e], p) < TOL


@pytest.mark.parametrize("wt,order", [(1, 2), (0, 1), (2, 0)])
def test_color_flow_batch_equals_one_ensemble_at_a_time(capi, ctx, torch, wt, order):
    """The batched call (one wall-filter, one flow and one gate launch per
    chunk of ensembles) gives every map of every ensemble bit for bit as the
    one-ensemble call does: lengths from 2 to 64 frames, ensembles that share
    frames, enough distinct lengths to split the projector pool (64, 40 and
    30 frames) and more ensembles than one launch takes (70)."""
    rng = np.random.default_rng(5)
    n0, n1, n_all = 6, 40, 64
    ph = np.exp(-1j * 0.35 * np.arange(n_all))[:, None, None] * np.exp(-1j * 0.85 * np.arange(n1))[None, None, :]
    noise = rng.normal(size=(n_all, n0, n1)) + 1j * rng.normal(size=(n_all, n0, n1))
    ens = (8.0 * np.exp(0.02j * np.arange(n_all))[:, None, None] + 2.0 * ph + 0.2 * noise).astype(np.complex64)
    ens[:, :, :10] *= 0.01
    d = dev(torch, ens)
    axis1 = np.linspace(0.02, 0.03, n1).astype(np.float32)
    cfg = capi.doppler_config(wall_filter=wt, polynomial_order=order)
    lens = [2, 5, 64, 40, 30, 7, 12] + [3] * 63
    offs = [int(rng.integers(0, n_all - n + 1)) for n in lens]
    m = len(lens)
    vel, pwr, var = (torch.empty((m, n0, n1), dtype=torch.float32, device="cuda") for _ in range(3))
    valid = torch.empty((m, n0, n1), dtype=torch.uint8, device="cuda")
    ctx.color_flow_batch(d.data_ptr(), lens, offs, n0, n1, axis1, 5e6, 5000.0, 1540.0, cfg, vel.data_ptr(),
                         pwr.data_ptr(), var.data_ptr(), valid.data_ptr())
    got = [host(torch, t) for t in (vel, pwr, var, valid)]
    one = [torch.empty((n0, n1), dtype=torch.float32, device="cuda") for _ in range(3)]
    one.append(torch.empty((n0, n1), dtype=torch.uint8, device="cuda"))
    for e, (n, o) in enumerate(zip(lens, offs)):
        sub = d[o:o + n].contiguous()
        ctx.color_flow(sub.data_ptr(), n, n0, n1, axis1, 5e6, 5000.0, 1540.0, cfg, *[t.data_ptr() for t in one])
        for g, w in zip(got, one):
            assert np.array_equal(g[e], host(torch, w)), (e, n)
    assert got[3].sum() > 0


def test_displacement_and_strain_match_reference(capi, ctx, torch, golden):
    g = golden("doppler")
    a, b = g["disp_a"], g["disp_b"]
    n0, n1 = a.shape
    ax = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    cr = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    da, db = dev(torch, a), dev(torch, b)
    ctx.axial_displacement(da.data_ptr(), db.data_ptr(), n0, n1, g["disp_ax1"], 5e6, 1540.0, 4, 1, 5,
                           ax.data_ptr(), cr.data_ptr())
    assert rel_l2(host(torch, ax), g["disp_axial"]) < TOL
    assert rel_l2(host(torch, cr), g["disp_corr"]) < TOL
    st = torch.empty((n0, n1), dtype=torch.float32, device="cuda")
    dax = dev(torch, g["disp_axial"])
    ctx.axial_strain(dax.data_ptr(), n0, n1, g["disp_ax1"], 9, st.data_ptr())
    assert rel_l2(host(torch, st), g["strain"]) < TOL


# ------------------------------------------------ full-size, size-independent

def test_full_size_das_is_linear_and_matches_oracle_on_lines(capi, ctx, torch, oracle):
    """75 plane waves, 128 channels, 512 x 1024 pixels: the frame is linear in
    the IQ data (checked on random inputs), and a sample of lines matches the
    oracle exactly as at small sizes."""
    pr = O.probe()
    med = O.medium()
    acq = O.acquisition(fs=20e6, n_samples=2073, prf=5000.0)
    ang = np.deg2rad(np.linspace(-16, 16, 75)).astype(np.float32)
    n_el = 128
    ex = ((np.arange(n_el, dtype=np.float32) - np.float32(0.5 * (n_el - 1))) * np.float32(300e-6)).astype(np.float32)
    delays = (ex[None, :] * np.sin(ang)[:, None] / np.float32(1540.0)).astype(np.float32)
    apod = np.ones((75, n_el), np.float32)
    txs = O.TxSet(np.ones(75, np.int32), ang, np.tile([0, 0, 0.03], (75, 1)).astype(np.float32),
                  np.zeros((75, 3), np.float32), delays, apod)
    rng = np.random.default_rng(3)
    shape = (75, n_el, 2073)
    x = (rng.standard_normal(shape, dtype=np.float32) + 1j * rng.standard_normal(shape, dtype=np.float32)).astype(np.complex64)
    y = (rng.standard_normal(shape, dtype=np.float32) + 1j * rng.standard_normal(shape, dtype=np.float32)).astype(np.complex64)
    half = 0.5 * (127 * 300e-6 + 270e-6)
    ax0 = np.linspace(-half, half, 512).astype(np.float32)
    ax1 = np.linspace(0.005, 0.060, 1024).astype(np.float32)
    pts = np.stack(np.meshgrid(ax0, [0.0], ax1, indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    ch = c_channel(capi, pr, med, acq, txs, is_iq=True, fdem=5e6)
    grid = capi.Grid(0, ax0, ax1, pts)
    plan = ctx.plan(ch, grid, capi.bf_config(f_number=1.5))
    dx, dy = dev(torch, x), dev(torch, y)
    fx = torch.empty((512, 1024), dtype=torch.complex64, device="cuda")
    fy = torch.empty_like(fx)
    fz = torch.empty_like(fx)
    plan.execute(dx.data_ptr(), fx.data_ptr())
    plan.execute(dy.data_ptr(), fy.data_ptr())
    dz = (2.0 * dx - 0.5j * dy).contiguous()
    plan.execute(dz.data_ptr(), fz.data_ptr())
    lin = 2.0 * fx - 0.5j * fy
    assert rel_l2(host(torch, fz), host(torch, lin)) < 1e-5
    lines = [0, 100, 255, 511]
    sub = pts.reshape(512, 1024, 3)[lines].reshape(-1, 3)
    want = oracle.beamform(O.channel_desc(pr, med, acq, txs, is_iq=True, fdem=5e6), x, sub, len(lines), 1024,
                           O.bf_config(f_number=1.5))
    got = host(torch, fx)[lines]
    assert rel_l2(got, want) < TOL
    plan.close()


def test_postprocess_empty_and_invalid_sizes(capi, ctx, torch):
    """Empty element counts are no-ops where the reference's loops simply do
    not run (TGC, log compression, maximum); an empty frame or raster, or a
    grid without samples, is an invalid argument (ValueError), and nothing
    is written."""
    buf = torch.full((64,), 3.0, device="cuda")
    out = torch.full((64,), 7.0, device="cuda")
    pts = torch.zeros((64, 3), device="cuda")
    ctx.apply_tgc(buf.data_ptr(), 0, 64, pts.data_ptr(), 0.5, 5e6, out.data_ptr())
    ctx.log_compress(buf.data_ptr(), 0, 60.0, 0.0, 0.0, out.data_ptr())
    assert bool((out == 7.0).all())
    with pytest.raises(ValueError):
        ctx.envelope(buf.data_ptr(), 0, 8, 5e6, out.data_ptr())
    ax = np.linspace(0.0, 0.01, 8, dtype=np.float32)
    p = np.zeros((64, 3), np.float32)
    p[:, 0] = np.repeat(ax, 8)
    p[:, 2] = np.tile(ax, 8)
    grid = capi.Grid(0, ax, ax, p)
    with pytest.raises(ValueError):
        ctx.scan_convert(buf.data_ptr(), grid, 0, 10, 0.0, out.data_ptr())
    with pytest.raises(ValueError):
        ctx.scan_convert(buf.data_ptr(), grid, 10, 0, 0.0, out.data_ptr())
    torch.cuda.synchronize()
    assert bool((out == 7.0).all())
