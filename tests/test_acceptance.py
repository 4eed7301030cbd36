"""The reference's Python acceptance scenarios (tests/test_usx.py of the
reference), run against this engine's `usx` module on the GPU: a user's
scripts written against the reference must behave the same here. Each test
names the scenario it restates; the thresholds are the reference's. The
host-only scenarios (probe geometry, acquisition depth, gCNR invariance) are
in tests/test_host.py. Also here: the simulated source and the device feed
of usx.ingest.
"""

from __future__ import annotations

import numpy as np
import pytest

import usx
from usx import ingest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    """64-element 5 MHz linear array, 40 mm acquisition, no noise
    (test_usx.py:17-26)."""
    probe = usx.presets.linear_5mhz()
    probe.n_elements = 64
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.04, medium=medium)
    cfg = usx.SimulatorConfig()
    cfg.noise_db = -200.0
    return probe, medium, acq, usx.Simulator(probe, medium, acq, cfg), cfg


def _envelope(iq, grid, cfg=None):
    bf = usx.Beamformer(cfg) if cfg is not None else usx.Beamformer()
    return np.asarray(usx.envelope(bf.beamform(iq, grid)))


def test_rf_is_a_view_of_the_engine_buffer(setup):
    """test_usx.py:48-58: ChannelData.rf is a writable float32 view."""
    probe, medium, acq, sim, _ = setup
    cd = sim.simulate(sim.make_plane_waves([0.0]), usx.Phantom.point_targets([usx.Vec3(0, 0, 0.02)]))
    rf = cd.rf
    assert rf.dtype == np.float32 and rf.shape == (1, probe.n_elements, acq.n_samples)
    rf[0, 0, 0] = -777.0
    assert float(cd.rf[0, 0, 0]) == -777.0
    assert not rf.flags.owndata


def test_pipeline_frame_is_complex_and_peaks_at_the_target(setup):
    """test_usx.py:61-72: the frame keeps phase and its envelope peaks within
    0.2 mm of a point target, in both axes."""
    probe, medium, acq, sim, _ = setup
    tx, tz = 0.004, 0.025
    cd = sim.simulate(sim.make_plane_waves([0.0]), usx.Phantom.point_targets([usx.Vec3(tx, 0.0, tz)]))
    grid = usx.ScanGrid.cartesian(0.0, 0.008, 81, 0.021, 0.029, 81)
    data = usx.ImagingPipeline(grid).process_frame(cd).data
    assert data.dtype == np.complex64
    i, j = np.unravel_index(np.abs(data).argmax(), data.shape)
    assert abs(float(np.asarray(grid.axis0)[i]) - tx) <= 2e-4
    assert abs(float(np.asarray(grid.axis1)[j]) - tz) <= 2e-4


def test_bmode_lies_in_unit_range(setup):
    """test_usx.py:75-84: to_bmode maps to [0, 1] with the brightest wire near 1."""
    probe, medium, acq, sim, _ = setup
    cd = sim.simulate(sim.make_plane_waves([0.0]), usx.phantoms.wire_targets(depths=(0.02, 0.03), lateral=(0.0,)))
    grid = usx.grid_for(probe, 0.01, 0.04, 64, 160)
    img = np.asarray(usx.to_bmode(usx.ImagingPipeline(grid).process_frame(cd), dynamic_range_db=50))
    assert img.shape == (64, 160)
    assert 0.0 <= img.min() and img.max() <= 1.0 and img.max() > 0.9


def test_compounding_narrows_the_point_spread(setup):
    """test_usx.py:87-104: 11 compounded plane waves over +-12 degrees give a
    lateral FWHM under 0.75 x that of one plane wave."""
    probe, medium, acq, sim, _ = setup
    ph = usx.Phantom.point_targets([usx.Vec3(0.0, 0.0, 0.025)])
    grid = usx.ScanGrid.cartesian(-0.004, 0.004, 161, 0.023, 0.027, 81)
    fwhm = {}
    for n in (1, 11):
        iq = usx.demodulate(sim.simulate(usx.presets.plane_wave_sequence(sim, 12.0, n), ph), usx.DemodConfig())
        env = _envelope(iq, grid, usx.BeamformerConfig())
        fwhm[n] = usx.metrics.measure_psf(env, grid, (0.0, 0.025)).lateral_fwhm
    assert fwhm[11] < 0.75 * fwhm[1], fwhm


def test_speckle_is_rayleigh(setup):
    """test_usx.py:131-143: fully developed speckle has mu / sigma = 1.91 (15%)."""
    probe, medium, acq, sim, _ = setup
    ph = usx.phantoms.cyst_phantom(probe, medium, cysts=(), z_min=0.010, z_max=0.035, density_per_cell=15.0)
    iq = usx.demodulate(sim.simulate(usx.presets.plane_wave_sequence(sim, 9.0, 5), ph), usx.DemodConfig())
    grid = usx.grid_for(probe, 0.015, 0.030, 96, 240)
    snr = usx.metrics.speckle_snr(_envelope(iq, grid), grid, (0.0, 0.0225), (0.005, 0.005))
    assert abs(snr - usx.metrics.RAYLEIGH_SPECKLE_SNR) <= 0.15 * usx.metrics.RAYLEIGH_SPECKLE_SNR, snr


def test_anechoic_cyst_is_dark_and_separable(setup):
    """test_usx.py:146-156: a 3 mm anechoic cyst is > 6 dB darker than the
    background with gCNR > 0.5."""
    probe, medium, acq, sim, _ = setup
    ph = usx.phantoms.cyst_phantom(probe, medium, cysts=((0.0, 0.025, 0.003, 0.0),), z_min=0.010, z_max=0.038)
    iq = usx.demodulate(sim.simulate(usx.presets.plane_wave_sequence(sim, 9.0, 7), ph), usx.DemodConfig())
    grid = usx.grid_for(probe, 0.015, 0.035, 128, 240)
    stats = usx.metrics.summarize(_envelope(iq, grid), grid, lesion_xz=(0.0, 0.025), lesion_radius=0.003)
    assert stats["contrast_db"] < -6.0 and stats["gcnr"] > 0.5, stats


def test_recorded_and_simulated_sources_beamform_alike(tmp_path, setup):
    """test_usx.py:159-185: a simulated source's frame written with save_npz
    and replayed by FileSource keeps samples and geometry, and beamforms to
    the same image (rtol 1e-5)."""
    probe, medium, acq, sim, cfg = setup
    txs = sim.make_plane_waves([0.0])
    ph = usx.phantoms.wire_targets(depths=(0.025,), lateral=(0.0,))
    frames = list(ingest.SimulatedSource(probe, medium, acq, ph, txs, config=cfg, n_frames=2).frames())
    assert len(frames) == 2
    rep = next(ingest.FileSource(ingest.save_npz(tmp_path / "acq.npz", frames[0])).frames())
    assert np.array_equal(np.asarray(frames[0].rf), np.asarray(rep.rf))
    assert rep.probe.n_elements == probe.n_elements
    assert rep.acq.sampling_frequency == pytest.approx(acq.sampling_frequency)
    assert len(rep.transmits) == 1 and np.allclose(rep.transmits[0].delays, txs[0].delays, atol=1e-12)
    grid = usx.ScanGrid.cartesian(-0.004, 0.004, 41, 0.022, 0.028, 61)
    a = _envelope(usx.demodulate(frames[0], usx.DemodConfig()), grid)
    b = _envelope(usx.demodulate(rep, usx.DemodConfig()), grid)
    assert np.allclose(a, b, rtol=1e-5, atol=1e-6)


def test_simulated_source_carries_motion_across_frames(setup):
    """Moving scatterers advance by velocity x (events / PRF) per frame
    (reference ingest.py:85-108): frame 1 equals a simulation of the displaced
    phantom."""
    probe, medium, acq, sim, cfg = setup
    txs = sim.make_plane_waves([0.0, 4.0])
    ph = usx.Phantom.point_targets([usx.Vec3(0.0, 0.0, 0.02), usx.Vec3(0.002, 0.0, 0.025)])
    ph.velocities = np.array([[0.0, 0.0, 0.3], [0.1, 0.0, -0.2]], np.float32)
    f = list(ingest.SimulatedSource(probe, medium, acq, ph, txs, config=cfg, n_frames=2).frames())
    moved = usx.Phantom()
    moved.extend(ph)
    moved.positions = (np.asarray(ph.positions, np.float64)
                       + np.asarray(ph.velocities, np.float64) * (len(txs) / acq.prf)).astype(np.float32)
    want = np.asarray(sim.simulate(txs, moved).rf)
    assert not np.array_equal(np.asarray(f[0].rf), np.asarray(f[1].rf))
    assert np.array_equal(np.asarray(f[1].rf), want)


def test_array_source_passes_blocks_through(setup):
    """test_usx.py:194-203."""
    probe, medium, acq, sim, _ = setup
    txs = sim.make_plane_waves([0.0])
    raw = np.asarray(sim.simulate(txs, usx.phantoms.wire_targets(depths=(0.025,), lateral=(0.0,))).rf).copy()
    got = list(ingest.ArraySource([raw, raw], probe, medium, acq, txs).frames())
    assert len(got) == 2 and np.array_equal(np.asarray(got[0].rf), raw)


def _flow(sim, acq, medium, velocity):
    ph = usx.Phantom.speckle_box(-0.006, 0.006, 0.022, 0.028, 1e-4, 3000, 5)
    ph.velocities = np.tile(np.asarray(velocity, np.float32), (len(ph), 1))
    iq = usx.demodulate(sim.simulate(usx.Simulator.repeat(sim.make_plane_waves([0.0]), 12), ph),
                        usx.DemodConfig())
    grid = usx.ScanGrid.cartesian(-0.003, 0.003, 21, 0.023, 0.027, 61)
    frames = usx.Beamformer().beamform_sequence(iq, grid, 1)
    cfg = usx.DopplerConfig()
    cfg.wall_filter = usx.WallFilter.NONE
    flow = usx.color_flow(frames, acq.prf, medium.speed_of_sound, cfg)
    valid = np.asarray(flow.valid).astype(bool)
    return flow, np.asarray(flow.velocity)[valid], valid


def test_doppler_measures_an_axial_velocity(setup):
    """test_usx.py:206-224: 0.12 m/s axial motion reads 0.12 +- 0.02 m/s."""
    probe, medium, acq, sim, _ = setup
    flow, v, valid = _flow(sim, acq, medium, (0.0, 0.0, 0.12))
    assert valid.sum() > 50
    assert abs(float(np.median(v)) - 0.12) <= 0.02
    assert flow.nyquist_velocity > 0.12


def test_doppler_ignores_lateral_motion(setup):
    """test_usx.py:227-242: 0.2 m/s lateral motion reads under 0.02 m/s."""
    probe, medium, acq, sim, _ = setup
    _, v, _ = _flow(sim, acq, medium, (0.20, 0.0, 0.0))
    assert abs(float(np.median(v))) < 0.02


def test_sector_scan_conversion_fills_the_sector():
    """test_usx.py:245-252."""
    grid = usx.ScanGrid.sector(-0.6, 0.6, 48, 0.01, 0.08, 96, usx.Vec3(0, 0, 0))
    px = np.asarray(usx.scan_convert(np.ones((48, 96), np.float32), grid, 160, 200, -1.0).pixels)
    assert px.shape == (200, 160)
    assert (px > 0.99).sum() > 3000 and (px < -0.5).sum() > 1000


def test_display_reference_settles_and_resets(setup):
    """test_usx.py:255-269: the same frame twice gives the same display; the
    pipeline counts frames, times them and resets."""
    probe, medium, acq, sim, _ = setup
    cd = sim.simulate(sim.make_plane_waves([0.0]), usx.phantoms.wire_targets(depths=(0.025,), lateral=(0.0,)))
    pipe = usx.ImagingPipeline(usx.grid_for(probe, 0.015, 0.035, 48, 120))
    a = np.asarray(pipe.process_display(cd))
    b = np.asarray(pipe.process_display(cd))
    assert pipe.frame_count == 2 and pipe.stats.total_ms > 0
    assert np.allclose(a, b, atol=1e-6)
    pipe.reset()
    assert pipe.frame_count == 0


@pytest.mark.parametrize("depth", [1, 2, 3])
def test_device_feed_delivers_every_frame_intact(setup, depth):
    """Frames arrive on the device in order and intact although the consumer
    overwrites each one on its stream right after using it (the slot is
    refilled only behind that work)."""
    import torch
    probe, medium, acq, sim, _ = setup
    txs = sim.make_plane_waves([-3.0, 0.0, 3.0])
    rng = np.random.default_rng(depth)
    blocks = [rng.standard_normal((3, probe.n_elements, acq.n_samples)).astype(np.float32) for _ in range(7)]
    stream = torch.cuda.Stream()
    sums = []
    feed = ingest.DeviceFeed(ingest.ArraySource(blocks, probe, medium, acq, txs), depth=depth, stream=stream)
    with torch.cuda.stream(stream):
        for fr in feed:
            assert fr.index == len(sums)
            sums.append(fr.rf.double().sum(dim=(1, 2)))
            fr.rf.mul_(0.0)
    torch.cuda.synchronize()
    assert len(sums) == len(blocks)
    for s, b in zip(sums, blocks):
        assert np.allclose(s.cpu().numpy(), b.astype(np.float64).sum(axis=(1, 2)), rtol=1e-9, atol=1e-9)


def test_device_feed_into_a_device_plan_matches_the_host_path(setup):
    """Frames streamed by the feed, demodulated and beamformed on the
    context's stream through the C-ABI, equal the host API's result."""
    import torch
    from usx import capi
    probe, medium, acq, sim, cfg = setup
    txs = sim.make_plane_waves([-2.0, 2.0])
    ph = usx.phantoms.wire_targets(depths=(0.02, 0.03), lateral=(0.0,))
    src = ingest.SimulatedSource(probe, medium, acq, ph, txs, config=cfg, n_frames=3)
    grid = usx.ScanGrid.cartesian(-0.004, 0.004, 33, 0.018, 0.032, 96)
    want = [np.asarray(usx.Beamformer().beamform(usx.demodulate(f, usx.DemodConfig()), grid).data)
            for f in src.frames()]
    ctx = capi.Context(0)
    tx = [dict(type=1, angle=t.angle, delays=t.delays, apodization=t.apodization) for t in txs]
    c_probe = capi.Probe(probe.n_elements, probe.pitch, probe.element_width, probe.elevation_height,
                         probe.center_frequency, probe.bandwidth)
    c_med = capi.Medium(medium.speed_of_sound, medium.attenuation, medium.density)
    c_acq = capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf)
    ch_rf = capi.Channel(c_probe, c_med, c_acq, tx)
    ch_iq = capi.Channel(c_probe, c_med, c_acq, tx, is_iq=True, fdem=probe.center_frequency)
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), np.asarray(grid.points).reshape(-1, 3))
    plan = ctx.plan(ch_iq, cgrid, capi.bf_config())
    iq = torch.empty((len(txs), probe.n_elements, acq.n_samples), dtype=torch.complex64, device="cuda")
    out = [torch.empty((33, 96), dtype=torch.complex64, device="cuda") for _ in want]
    for fr in ingest.DeviceFeed(src, depth=2, stream=ctx):
        ctx.demodulate(ch_rf, capi.demod_config(), fr.rf.data_ptr(), iq.data_ptr())
        plan.execute(iq.data_ptr(), out[fr.index].data_ptr())
    ctx.synchronize()
    for o, w in zip(out, want):
        got = o.cpu().numpy()
        assert np.linalg.norm(got - w) <= 1e-5 * np.linalg.norm(w)
    plan.close()
    ctx.close()


def test_device_feed_rejects_a_frame_of_another_shape(setup):
    """A feed carries frames of one shape: a source that changes shape mid-way
    raises ValueError at that frame, after delivering the frames before it."""
    import torch
    probe, medium, acq, sim, _ = setup
    txs = sim.make_plane_waves([0.0])
    a = np.ones((1, probe.n_elements, acq.n_samples), np.float32)

    class Ragged(ingest.ArraySource):
        def frames(self):
            yield from super().frames()
            yield usx.ChannelData.from_rf(np.ones((2, probe.n_elements, acq.n_samples), np.float32), probe,
                                          medium, acq, list(txs) * 2)

    feed = ingest.DeviceFeed(Ragged([a, a], probe, medium, acq, txs), depth=1)
    got = []
    with pytest.raises(ValueError, match="shape"):
        for fr in feed:
            got.append(float(fr.rf.sum()))
    torch.cuda.synchronize()
    assert got == [float(a.sum())] * 2
