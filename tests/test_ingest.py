"""Raw-data sources (usx.ingest) on the host: the array adapter, the .npz
recording round trip for every transmit type, multi-frame recordings and
looping, and the recording's key set, which is the reference's layout
(python/usx/ingest.py:201-233 of the reference) so that recordings move
between the two engines. The device feed and the simulated source need a GPU
and are covered in tests/test_acceptance.py."""

from __future__ import annotations

import numpy as np
import pytest

import usx
from usx import ingest

RECORDING_KEYS = {
    "rf", "probe_n_elements", "probe_pitch", "probe_element_width", "probe_elevation_height",
    "probe_center_frequency", "probe_bandwidth", "medium_speed_of_sound", "medium_attenuation",
    "acq_sampling_frequency", "acq_n_samples", "acq_t0", "acq_prf", "tx_type", "tx_angle", "tx_focus",
    "tx_origin", "tx_delays", "tx_apodization",
}


@pytest.fixture(scope="module")
def geometry():
    probe = usx.presets.linear_5mhz()
    probe.n_elements = 32
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.02, medium=medium)
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    txs = (list(sim.make_plane_waves([-4.0, 0.0]))
           + list(sim.make_focused_scan(2, -0.003, 0.003, 0.015))
           + list(sim.make_diverging_waves([0.0], 0.01)))
    return probe, medium, acq, txs


def _blocks(acq, txs, n, seed=0):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal((len(txs), 32, acq.n_samples)).astype(np.float32) for _ in range(n)]


def test_array_source_yields_the_blocks(geometry):
    probe, medium, acq, txs = geometry
    blocks = _blocks(acq, txs, 3)
    with ingest.ArraySource(blocks, probe, medium, acq, txs) as src:
        assert src.events_per_frame == len(txs)
        got = [np.asarray(cd.rf) for cd in src]
    assert len(got) == 3
    for a, b in zip(got, blocks):
        assert np.array_equal(a, b)


def test_recording_round_trip_keeps_samples_and_geometry(tmp_path, geometry):
    probe, medium, acq, txs = geometry
    cd = next(ingest.ArraySource(_blocks(acq, txs, 1), probe, medium, acq, txs).frames())
    path = ingest.save_npz(tmp_path / "rec.npz", cd)
    with np.load(path) as z:
        assert set(z.files) == RECORDING_KEYS
        assert list(z["tx_type"]) == [1, 1, 0, 0, 2]
    rep = next(ingest.FileSource(path).frames())
    assert np.array_equal(np.asarray(rep.rf), np.asarray(cd.rf))
    assert rep.probe.n_elements == probe.n_elements
    assert rep.probe.pitch == pytest.approx(probe.pitch)
    assert rep.probe.center_frequency == pytest.approx(probe.center_frequency)
    assert rep.medium.speed_of_sound == pytest.approx(medium.speed_of_sound)
    assert rep.acq.sampling_frequency == pytest.approx(acq.sampling_frequency)
    assert rep.acq.n_samples == acq.n_samples
    assert rep.acq.t0 == pytest.approx(acq.t0)
    assert len(rep.transmits) == len(txs)
    for a, b in zip(rep.transmits, txs):
        assert a.type == b.type
        assert a.angle == pytest.approx(b.angle)
        assert (a.focus.x, a.focus.z) == pytest.approx((b.focus.x, b.focus.z))
        assert (a.origin.x, a.origin.z) == pytest.approx((b.origin.x, b.origin.z))
        assert np.allclose(a.delays, b.delays, atol=1e-12, rtol=1e-6)
        assert np.allclose(a.apodization, b.apodization)


def test_multi_frame_recording_and_looping(tmp_path, geometry):
    """A recording whose rf holds several frames' events (frames x events,
    channels, samples) replays as one frame per block; loop=True cycles."""
    probe, medium, acq, txs = geometry
    blocks = _blocks(acq, txs, 3, seed=5)
    cd = next(ingest.ArraySource(blocks[:1], probe, medium, acq, txs).frames())
    one = ingest.save_npz(tmp_path / "one.npz", cd)
    with np.load(one) as z:
        arrays = {k: z[k] for k in z.files}
    arrays["rf"] = np.concatenate(blocks)
    np.savez_compressed(tmp_path / "cine.npz", **arrays)
    frames = [np.asarray(f.rf) for f in ingest.FileSource(tmp_path / "cine.npz").frames()]
    assert len(frames) == 3
    for a, b in zip(frames, blocks):
        assert np.array_equal(a, b)
    it = ingest.FileSource(tmp_path / "cine.npz", loop=True).frames()
    seen = [np.asarray(next(it).rf) for _ in range(7)]
    assert np.array_equal(seen[6], blocks[0]) and np.array_equal(seen[4], blocks[1])


@pytest.mark.skipif(__import__("torch").cuda.is_available(), reason="checks the no-GPU error")
def test_device_feed_fails_loudly_without_a_gpu(geometry):
    probe, medium, acq, txs = geometry
    with pytest.raises(RuntimeError, match="no CPU path"):
        ingest.DeviceFeed(ingest.ArraySource(_blocks(acq, txs, 1), probe, medium, acq, txs))
