"""Parity at the five benchmark configurations' own shapes (GPU against the
CPU oracle, whose FP32 restatement is bit-exact with the reference's build on
the golden fixtures).

The oracle runs on a subset where the full configuration would take minutes
on the host: each test's docstring says which. Seeded phantoms and transmit
tables come from this engine's host code (pinned to the reference's draw
order by tests/test_host.py) and feed both sides.

Tolerances (relative L2 unless stated), as in tests/test_gpu_parity.py:
  FP32 paths                      <= 1e-5
  minimum variance, FP32 solver   <= 1e-4
  minimum variance, tensor cores  <= 1e-3
  image metrics (CNR, gCNR, speckle SNR, lateral and axial FWHM): each
  within 1% of the oracle frame's value.
"""

from __future__ import annotations

import os

import numpy as np
import pytest

import configs as CF
from gold import rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-5
TOL_MV = 1e-4
TOL_MV_TC = 1e-3


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


@pytest.fixture(scope="module")
def orc(oracle):
    oracle.set_threads(os.cpu_count() or 1)
    return oracle


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(torch, t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gpu_rf_iq(capi, ctx, torch, s, sc, noise_db=-200.0, enable_motion=1):
    """Simulate and demodulate on the device; (RF, IQ) device tensors."""
    n_ev, n_el, n_smp = len(s.txs), s.probe.n_elements, s.acq.n_samples
    ch = CF.capi_channel(capi, s)
    d_sc = dev(torch, sc)
    rf = torch.empty((n_ev, n_el, n_smp), dtype=torch.float32, device="cuda")
    iq = torch.empty((n_ev, n_el, n_smp), dtype=torch.complex64, device="cuda")
    ctx.simulate(ch, capi.sim_config(noise_db=noise_db, enable_motion=enable_motion), d_sc.data_ptr(), len(sc),
                 None, rf.data_ptr())
    fdem = ctx.demodulate(ch, capi.demod_config(), rf.data_ptr(), iq.data_ptr())
    assert fdem == pytest.approx(s.probe.center_frequency)
    return rf, iq


def gpu_frame(capi, ctx, torch, s, iq, grid_pts, n0, n1, kw, gtype=0, mv_mode=None, axes=None):
    ch = CF.capi_channel(capi, s, is_iq=True, fdem=s.probe.center_frequency)
    ax0, ax1 = axes if axes is not None else (np.asarray(s.grid.axis0), np.asarray(s.grid.axis1))
    grid = capi.Grid(gtype, ax0, ax1, np.asarray(grid_pts, np.float32).reshape(-1, 3))
    plan = ctx.plan(ch, grid, capi.bf_config(**kw))
    if mv_mode is not None:
        plan.set_mv_mode(mv_mode)
    out = torch.empty((n0, n1), dtype=torch.complex64, device="cuda")
    plan.execute(iq.data_ptr(), out.data_ptr())
    got = host(torch, out)
    stats = plan.mv_stats() if mv_mode in (1, 2, 3) else None
    plan.close()
    return got, stats


# ---------------------------------------------------------------- config 1

@pytest.fixture(scope="module")
def cfg1_run(orc):
    """Config 1 through the public API (usx.Simulator -> usx.demodulate ->
    usx.Beamformer) and through the oracle, from the same phantom."""
    s = CF.cfg1()
    usx = s.usx
    raw = s.sim.simulate(s.txs, s.phantom)
    iq = usx.demodulate(raw)
    sc = CF.scatterers(s.phantom)
    cd = CF.o_channel(s)
    rf_o = orc.simulate(cd, O.sim_config(noise_db=-200.0), sc)
    iq_o = orc.demodulate(cd, O.demod_config(), rf_o)
    cd_iq = CF.o_channel(s, is_iq=True, fdem=s.probe.center_frequency)
    pts = np.asarray(s.grid.points, np.float32).reshape(-1, 3)
    frames, frames_o, frames_stage = {}, {}, {}
    for name, kw in (("das", dict(f_number=1.5)), ("cf", dict(f_number=1.5, coherence_factor=1)),
                     ("dmas", dict(f_number=1.5, combiner=1))):
        bcfg = usx.BeamformerConfig()
        bcfg.f_number = 1.5
        if name == "cf":
            bcfg.coherence_factor = True
        if name == "dmas":
            bcfg.combiner = usx.Combiner.DMAS
        frames[name] = np.asarray(usx.Beamformer(bcfg).beamform(iq, s.grid).data)
        frames_o[name] = orc.beamform(cd_iq, iq_o, pts, 256, 640, O.bf_config(**kw))
        # The same stage from the GPU's own IQ: the beamformer alone against the oracle.
        frames_stage[name] = orc.beamform(cd_iq, np.asarray(iq.iq), pts, 256, 640, O.bf_config(**kw))
    return dict(s=s, raw=raw, iq=iq, rf_o=rf_o, iq_o=iq_o, frames=frames, frames_o=frames_o,
                frames_stage=frames_stage)


def test_cfg1_rf_iq_and_frames_match_oracle(cfg1_run):
    """11 plane waves, 20,000 scatterers, 128 x 1814 RF, 256 x 640 frames:
    RF, IQ and the DAS, coherence-factor and DMAS frames of the whole chain
    agree with the oracle's chain, and each beamformer agrees with the oracle
    on the GPU's own IQ."""
    r = cfg1_run
    assert np.asarray(r["raw"].rf).shape == (11, 128, 1814)
    assert rel_l2(np.asarray(r["raw"].rf), r["rf_o"]) < TOL
    assert rel_l2(np.asarray(r["iq"].iq), r["iq_o"]) < TOL
    for name in ("das", "cf", "dmas"):
        assert r["frames"][name].shape == (256, 640)
        assert rel_l2(r["frames"][name], r["frames_stage"][name]) < TOL, name
        assert rel_l2(r["frames"][name], r["frames_o"][name]) < TOL, name


def test_cfg1_image_metrics_within_one_percent(cfg1_run):
    """CNR and gCNR of the 3 mm cyst, speckle SNR of a background patch and
    the lateral and axial FWHM of all five wires, from the GPU frame and from
    the oracle's frame (reference metrics module, python/usx/metrics.py),
    agree within 1%. The reference's own checks on such a scene hold too:
    the wires sit where they were placed (core/tests/test_main.cpp:262-309,
    0.21 mm) and the anechoic cyst is more than 6 dB below the background
    (test_main.cpp:619-656)."""
    from usx import metrics as M
    r = cfg1_run
    s = r["s"]
    for name in ("das", "cf", "dmas"):
        env = np.abs(r["frames"][name])
        env_o = np.abs(r["frames_o"][name])
        got = CF.image_metrics(env, s.grid, CF.CFG1_CYST, CF.CFG1_WIRES, (0.008, 0.030))
        want = CF.image_metrics(env_o, s.grid, CF.CFG1_CYST, CF.CFG1_WIRES, (0.008, 0.030))
        for k, v in want.items():
            assert np.isfinite(v), (name, k)
            assert abs(got[k] - v) <= 0.01 * abs(v), (name, k, got[k], v)
    env = np.abs(r["frames"]["das"])
    for x, z in CF.CFG1_WIRES:
        psf = M.measure_psf(env, s.grid, (x, z))
        assert abs(psf.x - x) <= 2.1e-4 and abs(psf.z - z) <= 2.1e-4, (x, z, psf)
    assert M.contrast_db(env, s.grid, CF.CFG1_CYST[:2], CF.CFG1_CYST[2]) < -6.0


def test_cfg1_process_frame_and_display_match_oracle_chain(cfg1_run, orc):
    """usx.ImagingPipeline.process_frame on the RF acquisition equals the
    oracle's demodulation + beamforming of the same RF, and process_display
    equals the oracle's envelope -> TGC -> log compression against the
    pipeline's smoothed reference peak (core/src/pipeline.cpp:25-74), over
    two frames so the smoothing carries state."""
    r = cfg1_run
    s = r["s"]
    usx = s.usx
    pcfg = usx.PipelineConfig()
    pcfg.beamformer.f_number = 1.5
    pipe = usx.ImagingPipeline(s.grid, pcfg)
    frame = pipe.process_frame(r["raw"])
    cd_iq = CF.o_channel(s, is_iq=True, fdem=s.probe.center_frequency)
    pts = np.asarray(s.grid.points, np.float32).reshape(-1, 3)
    want = orc.beamform(cd_iq, orc.demodulate(CF.o_channel(s), O.demod_config(), np.asarray(r["raw"].rf)), pts,
                        256, 640, O.bf_config(f_number=1.5))
    assert rel_l2(np.asarray(frame.data), want) < TOL
    assert pipe.frame_count == 1
    # Display chain, two frames (the second at half amplitude moves the reference).
    pipe.reset()
    reference = 0.0
    a = np.float32(0.85)
    raw2 = usx.ChannelData.from_rf(np.asarray(r["raw"].rf) * np.float32(0.5), s.probe, s.medium, s.acq, s.txs)
    for raw in (r["raw"], raw2):
        img = np.asarray(pipe.process_display(raw))
        fr = orc.beamform(cd_iq, orc.demodulate(CF.o_channel(s), O.demod_config(), np.asarray(raw.rf)), pts,
                          256, 640, O.bf_config(f_number=1.5))
        env = orc.envelope(fr, s.probe.center_frequency)
        env = orc.apply_tgc(env, pts, s.medium.attenuation, s.probe.center_frequency)
        peak = np.float32(env.max())
        reference = peak if reference <= 0 else np.float32(a * np.float32(reference) + np.float32(1 - a) * peak)
        want_img = orc.log_compress(env, 60.0, 0.0, float(reference))
        assert img.shape == (256, 640)
        assert rel_l2(img, want_img) < TOL
        if raw is r["raw"]:
            first = want_img
    # to_display of a host frame takes the same device chain (frame uploaded once).
    pipe2 = usx.ImagingPipeline(s.grid, pcfg)
    img2 = np.asarray(pipe2.to_display(pipe2.process_frame(r["raw"]), s.medium))
    assert rel_l2(img2, first) < TOL


# ---------------------------------------------------------------- config 2

@pytest.fixture(scope="module")
def cfg2_run(capi, ctx, torch):
    s = CF.cfg2()
    sc = CF.scatterers(s.phantom)
    rf, iq = gpu_rf_iq(capi, ctx, torch, s, sc, noise_db=-60.0)
    return dict(s=s, sc=sc, rf=rf, iq=iq)


CFG2_LINES = np.linspace(0, 511, 16).round().astype(int)


def test_cfg2_simulator_100k_scatterers_matches_oracle(cfg2_run, capi, ctx, torch, orc):
    """The forward simulator at the full 100,000-scatterer phantom and 128
    elements, on three of the 75 plane waves (first, middle, last; the oracle
    needs about a second per transmit on the host), without noise."""
    r = cfg2_run
    s = r["s"]
    idx = [0, 37, 74]
    sub = [s.txs[i] for i in idx]
    ch = CF.capi_channel(capi, s, txs=sub)
    d_sc = dev(torch, r["sc"])
    rf = torch.empty((3, 128, s.acq.n_samples), dtype=torch.float32, device="cuda")
    ctx.simulate(ch, capi.sim_config(noise_db=-200.0), d_sc.data_ptr(), len(r["sc"]), None, rf.data_ptr())
    want = orc.simulate(CF.o_channel(s, txs=sub), O.sim_config(noise_db=-200.0), r["sc"])
    assert rel_l2(host(torch, rf), want) < TOL


@pytest.mark.parametrize("name,kw,tol", [
    ("das", dict(f_number=1.5), TOL),
    ("cf", dict(f_number=1.5, coherence_factor=1), TOL),
    ("dmas", dict(f_number=1.5, combiner=1), TOL),
])
def test_cfg2_plain_beamformers_on_full_lines(cfg2_run, capi, ctx, torch, orc, name, kw, tol):
    """75 plane waves, 128 channels, the simulated 100,000-scatterer phantom:
    16 full-depth lines (1024 samples each) spread over the 512-line grid
    against the oracle."""
    r = cfg2_run
    s = r["s"]
    pts = np.asarray(s.grid.points, np.float32).reshape(512, 1024, 3)[CFG2_LINES].reshape(-1, 3)
    axes = (np.asarray(s.grid.axis0)[CFG2_LINES], np.asarray(s.grid.axis1))
    got, _ = gpu_frame(capi, ctx, torch, s, r["iq"], pts, len(CFG2_LINES), 1024, kw, axes=axes)
    cd = CF.o_channel(s, is_iq=True, fdem=5e6)
    want = orc.beamform(cd, host(torch, r["iq"]), pts, len(CFG2_LINES), 1024, O.bf_config(**kw))
    assert rel_l2(got, want) < tol


MV64 = dict(f_number=1.5, combiner=2, mv_subarray=64, mv_diagonal_loading=0.01, mv_range_average=2)


def test_cfg2_minimum_variance_l64_on_full_lines(cfg2_run, capi, ctx, torch, orc):
    """Minimum variance at subarray 64, diagonal loading tr(R)/(100 L), range
    averaging +/-2 on 16 full-depth lines of the 75-PW acquisition against the
    oracle (the reference's combine_mv_windowed, core/src/beamformer.cpp:
    137-214): the reference-order FP32 solver and the FP32 lag-recurrence
    solver within 1e-4, the BF16 tensor-core covariances (tcgen05 and
    mma.sync) with refinement within 1e-3, with no failed refinement."""
    r = cfg2_run
    s = r["s"]
    pts = np.asarray(s.grid.points, np.float32).reshape(512, 1024, 3)[CFG2_LINES].reshape(-1, 3)
    axes = (np.asarray(s.grid.axis0)[CFG2_LINES], np.asarray(s.grid.axis1))
    cd = CF.o_channel(s, is_iq=True, fdem=5e6)
    iq_h = host(torch, r["iq"])
    want = orc.beamform(cd, iq_h, pts, len(CFG2_LINES), 1024, O.bf_config(**MV64))
    exact, _ = gpu_frame(capi, ctx, torch, s, r["iq"], pts, len(CFG2_LINES), 1024, MV64, mv_mode=0, axes=axes)
    assert rel_l2(exact, want) < TOL_MV
    tc, (fp64, failed) = gpu_frame(capi, ctx, torch, s, r["iq"], pts, len(CFG2_LINES), 1024, MV64, mv_mode=1,
                                   axes=axes)
    assert rel_l2(tc, want) < TOL_MV_TC
    assert failed == 0
    # The same solver with the covariance on warp-level mma.sync: the two
    # tensor-core covariances sum the same BF16 products in another order.
    mma, (_, failed2) = gpu_frame(capi, ctx, torch, s, r["iq"], pts, len(CFG2_LINES), 1024, MV64, mv_mode=2,
                                  axes=axes)
    assert rel_l2(mma, want) < TOL_MV_TC and failed2 == 0
    assert rel_l2(tc, mma) < 1e-4
    # FP32 covariance by the lag recurrence and one FP32 solve: the exact
    # solver's bar.
    f32, (fp64_3, failed3) = gpu_frame(capi, ctx, torch, s, r["iq"], pts, len(CFG2_LINES), 1024, MV64, mv_mode=3,
                                       axes=axes)
    assert rel_l2(f32, want) < TOL_MV and failed3 == 0 and fp64_3 == 0


# ---------------------------------------------------------------- config 4

@pytest.fixture(scope="module")
def cfg4_frames(capi, ctx, torch):
    """32 pulses x 3 plane waves of the flow phantom, beamformed as a
    sequence (one frame per pulse) onto 256 x 512 on the device."""
    s = CF.cfg4_doppler(32)
    sc = CF.cfg4_doppler_scatterers(s.phantom)
    rf, iq = gpu_rf_iq(capi, ctx, torch, s, sc)
    del rf
    ch = CF.capi_channel(capi, s, is_iq=True, fdem=5e6)
    grid = CF.capi_grid(capi, s.grid)
    plan = ctx.plan(ch, grid, capi.bf_config(f_number=1.5))
    frames = torch.empty((32, 256 * 512), dtype=torch.complex64, device="cuda")
    plan.execute_sequence(3, 32, iq.data_ptr(), frames.data_ptr(), 256 * 512)
    plan.close()
    return dict(s=s, iq=iq, frames=frames)


def test_cfg4_sequence_frames_match_oracle(cfg4_frames, torch, orc):
    """beamform_sequence of the Doppler acquisition: frames 0, 15 and 31
    (events 3f..3f+2) against the oracle's beamformer on those events."""
    r = cfg4_frames
    s = r["s"]
    iq_h = host(torch, r["iq"])
    f = host(torch, r["frames"]).reshape(32, 256, 512)
    pts = np.asarray(s.grid.points, np.float32).reshape(-1, 3)
    cd = CF.o_channel(s, is_iq=True, fdem=5e6)
    for k in (0, 15, 31):
        want = orc.beamform(cd, iq_h, pts, 256, 512, O.bf_config(f_number=1.5), 3 * k, 3 * k + 3)
        assert rel_l2(f[k], want) < TOL, k


def test_cfg4_color_flow_uneven_ensembles(cfg4_frames, capi, ctx, torch, orc):
    """Ensembles of 8, 12, 16 and 32 pulses packed into one batch call,
    order-2 polynomial wall filter and Loupas velocity, against the oracle's
    color_flow on each ensemble (core/src/doppler.cpp:77-176): power within
    1e-5, validity masks equal except at most 1% of pixels at a gate
    boundary, velocity within 1e-4 where both are valid."""
    r = cfg4_frames
    s = r["s"]
    lens = [8, 12, 16, 32]
    frames = r["frames"]
    packed = torch.cat([frames[:n] for n in lens]).contiguous()
    offs = np.cumsum([0] + lens[:-1])
    axis1 = np.asarray(s.grid.axis1)
    vel, pw, var = (torch.empty((4, 256 * 512), device="cuda") for _ in range(3))
    valid = torch.empty((4, 256 * 512), dtype=torch.uint8, device="cuda")
    dcfg = capi.doppler_config(wall_filter=1, polynomial_order=2, loupas=1)
    ctx.color_flow_batch(packed.data_ptr(), lens, offs, 256, 512, axis1, 5e6, 5000.0 / 3.0, 1540.0, dcfg,
                         vel.data_ptr(), pw.data_ptr(), var.data_ptr(), valid.data_ptr())
    V, P, S, M = (host(torch, t).reshape(4, 256, 512) for t in (vel, pw, var, valid))
    f_h = host(torch, frames).reshape(32, 256, 512)
    for e, n in enumerate(lens):
        v_o, p_o, s_o, m_o, _ = orc.color_flow(f_h[:n], axis1, 5e6, 5000.0 / 3.0, 1540.0,
                                               O.doppler_config(wall_filter=1, polynomial_order=2, loupas=1))
        assert rel_l2(P[e], p_o) < TOL, n
        assert np.mean(M[e] != m_o) <= 0.01, n
        both = (M[e] == 1) & (m_o == 1)
        assert both.sum() > 100, n
        assert rel_l2(V[e][both], v_o[both]) < 1e-4, n
        assert rel_l2(S[e][both], s_o[both]) < 1e-4, n


def _track_parity(got, want):
    """The integer lag search (core/src/doppler.cpp:234-261) may break a
    near-tie differently after a last-ulp difference in a correlation; such
    pixels (at most 0.1%) are excluded, the rest agree within 1e-5."""
    far = np.abs(got - want) > 1e-3 * np.abs(want).max()
    assert far.mean() <= 1e-3, far.mean()
    assert rel_l2(got[~far], want[~far]) < TOL


@pytest.mark.parametrize("max_lag", [8, 12])
def test_cfg4_displacement_and_strain_full_grid(capi, ctx, torch, orc, max_lag):
    """The elastography pair (4x stiff 5 mm inclusion at 30 mm, 1%
    compression), one plane wave, beamformed onto 256 x 1024 on the device:
    the two frames against the oracle, then axial displacement (kernel
    8 x 2, lag search +/-8 and +/-12 samples) and the least-squares strain
    over 2 mm against the oracle on the same frames."""
    s, phs = CF.cfg4_strain()
    pts = np.asarray(s.grid.points, np.float32).reshape(-1, 3)
    cd = CF.o_channel(s, is_iq=True, fdem=5e6)
    frames = []
    for ph in phs:
        _, iq = gpu_rf_iq(capi, ctx, torch, s, CF.scatterers(ph), enable_motion=0)
        got, _ = gpu_frame(capi, ctx, torch, s, iq, pts, 256, 1024, dict(f_number=1.5))
        want = orc.beamform(cd, host(torch, iq), pts, 256, 1024, O.bf_config(f_number=1.5))
        assert rel_l2(got, want) < TOL
        frames.append(got)
    axis1 = np.asarray(s.grid.axis1)
    dz = float(axis1[1] - axis1[0])
    fit = max(3, int(round(0.002 / dz)) | 1)
    da, db = dev(torch, frames[0]), dev(torch, frames[1])
    ax = torch.empty((256, 1024), device="cuda")
    cr = torch.empty_like(ax)
    ctx.axial_displacement(da.data_ptr(), db.data_ptr(), 256, 1024, axis1, 5e6, 1540.0, 8, 2, max_lag,
                           ax.data_ptr(), cr.data_ptr())
    want_ax, want_cr = orc.displacement(frames[0], frames[1], axis1, 5e6, 1540.0, 8, 2, max_lag)
    got_ax, got_cr = host(torch, ax), host(torch, cr)
    _track_parity(got_ax, want_ax)
    _track_parity(got_cr, want_cr)
    st = torch.empty_like(ax)
    d_want = dev(torch, want_ax)
    ctx.axial_strain(d_want.data_ptr(), 256, 1024, axis1, fit, st.data_ptr())
    assert rel_l2(host(torch, st), orc.strain(want_ax, axis1, fit)) < TOL
    # The inclusion is stiffer: less strain inside it than in the background.
    sm = orc.strain(want_ax, axis1, fit)
    x = np.asarray(s.grid.axis0)[:, None]
    z = axis1[None, :]
    inside = np.hypot(x, z - 0.030) < 0.003
    ring = (np.abs(x) < 0.004) & (np.abs(z - 0.020) < 0.003)
    assert np.median(np.abs(sm[inside])) < np.median(np.abs(sm[ring]))


# ---------------------------------------------------------------- config 5

@pytest.fixture(scope="module")
def cfg5_run(capi, ctx, torch):
    s = CF.cfg5_sector()
    sc = CF.scatterers(s.phantom)
    rf, iq = gpu_rf_iq(capi, ctx, torch, s, sc)
    return dict(s=s, sc=sc, rf=rf, iq=iq)


def test_cfg5_simulator_diverging_waves_matches_oracle(cfg5_run, capi, ctx, torch, orc):
    """64-element phased array, 100,000 scatterers, diverging waves: three of
    the 31 transmits (-45, 0 and +45 deg) against the oracle."""
    r = cfg5_run
    s = r["s"]
    sub = [s.txs[i] for i in (0, 15, 30)]
    ch = CF.capi_channel(capi, s, txs=sub)
    d_sc = dev(torch, r["sc"])
    rf = torch.empty((3, 64, s.acq.n_samples), dtype=torch.float32, device="cuda")
    ctx.simulate(ch, capi.sim_config(noise_db=-200.0), d_sc.data_ptr(), len(r["sc"]), None, rf.data_ptr())
    want = orc.simulate(CF.o_channel(s, txs=sub), O.sim_config(noise_db=-200.0), r["sc"])
    assert rel_l2(host(torch, rf), want) < TOL


def test_cfg5_sector_frame_and_scan_conversion(cfg5_run, capi, ctx, torch, orc):
    """31 diverging waves onto 256 beams x 1024 samples (the whole frame
    against the oracle), then envelope, 60 dB log compression and scan
    conversion to 800 x 800 against the oracle's chain on the same frame
    (core/src/postprocess.cpp:67-178)."""
    r = cfg5_run
    s = r["s"]
    pts = np.asarray(s.grid.points, np.float32).reshape(-1, 3)
    got, _ = gpu_frame(capi, ctx, torch, s, r["iq"], pts, 256, 1024, dict(f_number=1.5), gtype=1)
    cd = CF.o_channel(s, is_iq=True, fdem=2.5e6)
    iq_h = host(torch, r["iq"])
    want = orc.beamform(cd, iq_h, pts, 256, 1024, O.bf_config(f_number=1.5))
    assert rel_l2(got, want) < TOL
    ax0, ax1 = np.asarray(s.grid.axis0), np.asarray(s.grid.axis1)
    d_fr = dev(torch, got)
    env = torch.empty((256, 1024), device="cuda")
    logi = torch.empty_like(env)
    img = torch.empty((800, 800), device="cuda")
    ctx.envelope(d_fr.data_ptr(), 256, 1024, 2.5e6, env.data_ptr())
    ctx.log_compress(env.data_ptr(), 256 * 1024, 60.0, 0.0, -1.0, logi.data_ptr())
    grid = capi.Grid(1, ax0, ax1, pts)
    ext = ctx.scan_convert(logi.data_ptr(), grid, 800, 800, 0.0, img.data_ptr())
    env_o = orc.envelope(got, 2.5e6)
    log_o = orc.log_compress(env_o, 60.0, 0.0, -1.0)
    assert rel_l2(host(torch, logi), log_o) < TOL
    want_img, want_ext = orc.scan_convert(log_o, 1, ax0, ax1, (0, 0, 0), pts, 800, 800, 0.0)
    assert np.array_equal(ext, want_ext)
    assert rel_l2(host(torch, img), want_img) < TOL


def test_cfg5_sector_minimum_variance_tensor_cores(cfg5_run, capi, ctx, torch, orc):
    """Minimum variance (subarray 32) of the sector frame on the tensor cores,
    16 full-depth beams against the oracle within 1e-3."""
    r = cfg5_run
    s = r["s"]
    beams = np.linspace(0, 255, 16).round().astype(int)
    pts = np.asarray(s.grid.points, np.float32).reshape(256, 1024, 3)[beams].reshape(-1, 3)
    kw = dict(f_number=1.5, combiner=2, mv_subarray=32, mv_diagonal_loading=0.01, mv_range_average=2)
    axes = (np.asarray(s.grid.axis0)[beams], np.asarray(s.grid.axis1))
    got, (fp64, failed) = gpu_frame(capi, ctx, torch, s, r["iq"], pts, 16, 1024, kw, gtype=1, mv_mode=1, axes=axes)
    cd = CF.o_channel(s, is_iq=True, fdem=2.5e6)
    want = orc.beamform(cd, host(torch, r["iq"]), pts, 16, 1024, O.bf_config(**kw))
    assert rel_l2(got, want) < TOL_MV_TC
    assert failed == 0
