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


class _FakeCuda:
    """Records the stream operations DeviceFeed issues (no GPU involved)."""

    def __init__(self, log):
        self.log = log
        fake = self

        class Event:
            n = 0

            def __init__(self, *a, **k):
                Event.n += 1
                self.id = Event.n

            def record(self, stream):
                fake.log.append(("record", self.id, stream.name))

            def synchronize(self):
                fake.log.append(("host_wait", self.id))

        class Stream:
            def __init__(self, *a, name="copy", **k):
                self.name = name

            def wait_event(self, ev):
                fake.log.append(("wait", self.name, ev.id))

        class _Ctx:
            def __init__(self, s):
                self.s = s

            def __enter__(self):
                fake.current = self.s

            def __exit__(self, *a):
                fake.current = None

        self.Event, self.Stream = Event, Stream
        self.current = None
        self.stream = _Ctx

    def is_available(self):
        return True

    def current_device(self):
        return 0

    def current_stream(self, device=None):
        return self.Stream(name="consumer")


class _FakeTensor:
    def __init__(self, shape, log, kind):
        self.a = np.zeros(shape, np.float32)
        self.log, self.kind = log, kind

    def numpy(self):
        return self.a

    def copy_(self, src, non_blocking=False):
        self.a[...] = src.a
        self.log.append(("copy", int(src.a.flat[0])))

    def record_stream(self, s):
        pass


def test_device_feed_orders_copies_and_slot_reuse(monkeypatch, geometry):
    """With depth 2: frame k's copy waits for the consumer's release of its
    slot (recorded when the consumer asked for frame k - 1), each frame is
    handed over behind the event of its own copy, and the copies run ahead of
    the consumer by one frame."""
    import sys
    import types
    log = []
    cuda = _FakeCuda(log)
    fake = types.SimpleNamespace(
        cuda=cuda, float32=np.float32, device=lambda *a: "cuda:0",
        empty=lambda shape, dtype=None, pin_memory=False, device=None: _FakeTensor(
            shape, log, "host" if pin_memory else "device"))
    monkeypatch.setitem(sys.modules, "torch", fake)
    probe, medium, acq, txs = geometry
    blocks = [np.full((len(txs), 32, acq.n_samples), k, np.float32) for k in range(5)]
    feed = ingest.DeviceFeed(ingest.ArraySource(blocks, probe, medium, acq, txs), depth=2)
    seen = []
    for fr in feed:
        log.append(("consume", fr.index))
        seen.append(int(fr.rf.numpy().flat[0]))
    assert seen == [0, 1, 2, 3, 4]
    copies = [i for i, e in enumerate(log) if e[0] == "copy"]
    consumes = [i for i, e in enumerate(log) if e[0] == "consume"]
    assert [log[i][1] for i in copies] == [0, 1, 2, 3, 4]
    # Frame k + 1 is copied before frame k is consumed (one frame ahead).
    for k in range(4):
        assert copies[k + 1] < consumes[k]
    # Before copying frame k >= 2 into its slot, the copy stream waited on an
    # event the consumer recorded after consuming frame k - 2.
    for k in range(2, 5):
        waits = [i for i in range(consumes[k - 2], copies[k]) if log[i][0] == "wait" and log[i][1] == "copy"]
        assert waits, k
        ev = log[waits[-1]][2]
        rec = [i for i in range(consumes[k - 2], waits[-1]) if log[i] == ("record", ev, "consumer")]
        assert rec, k
    # The consumer waits on some copy event before each frame is handed over.
    for k in range(5):
        start = consumes[k - 1] if k else 0
        assert any(log[i][0] == "wait" and log[i][1] == "consumer" for i in range(start, consumes[k])), k
