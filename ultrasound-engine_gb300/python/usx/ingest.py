"""Sources of raw channel data, and the feed that streams them onto the GPU.

Every source answers two questions, as the reference's ingest protocol does
(python/usx/ingest.py:28-66 of the reference):

    metadata -> SourceMetadata(probe, medium, acquisition, transmits)
    frames() -> iterator of ChannelData, one per image frame

so the beamformer, the metrics and the display do not care whether a frame was
simulated (`SimulatedSource`), replayed from a self-describing `.npz`
recording (`FileSource`, written by `save_npz`) or handed over as arrays by a
scanner driver (`ArraySource`). The `.npz` layout keeps the reference's keys
(rf plus probe_*, medium_*, acq_*, tx_*), so recordings move between the two
engines unchanged.

`DeviceFeed` is what this engine adds on the GPU side: it stages each frame's
RF block in pinned host memory and copies it to device memory on a side
stream while the consumer's stream still works on the previous frames, so
the host-to-device copy leaves the critical path (depth slots in flight).
"""

from __future__ import annotations

import abc
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from ._usx import (Acquisition, ChannelData, Medium, Phantom, Probe, Simulator, SimulatorConfig, Transmit,
                   TransmitType, Vec3)

# Transmit types in the recording's integer code (reference ingest.py:187-189, 222).
_TX_TYPES = (TransmitType.FOCUSED, TransmitType.PLANE_WAVE, TransmitType.DIVERGING)


@dataclass
class SourceMetadata:
    """The geometry needed to interpret a source's frames."""

    probe: Probe
    medium: Medium
    acquisition: Acquisition
    transmits: list = field(default_factory=list)


class RawSource(abc.ABC):
    """A source of pre-beamforming channel data (one ChannelData per frame)."""

    @property
    @abc.abstractmethod
    def metadata(self) -> SourceMetadata:
        ...

    @abc.abstractmethod
    def frames(self):
        """Yield ChannelData objects, one per image frame."""

    def __iter__(self):
        return self.frames()

    @property
    def events_per_frame(self) -> int:
        return len(self.metadata.transmits)

    def close(self) -> None:
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class SimulatedSource(RawSource):
    """Frames synthesised from a phantom by the GPU simulator.

    `n_frames=None` streams without end. Moving scatterers carry their motion
    across frames: frame i simulates the phantom displaced by
    velocity * i * (events per frame / PRF), so a stream is continuous in time
    (reference ingest.py:69-108).
    """

    def __init__(self, probe: Probe, medium: Medium, acquisition: Acquisition, phantom: Phantom,
                 transmits: list, config: SimulatorConfig | None = None, n_frames: int | None = 1):
        self._sim = Simulator(probe, medium, acquisition, config or SimulatorConfig())
        self._meta = SourceMetadata(probe, medium, acquisition, list(transmits))
        self._phantom = phantom
        self._n_frames = n_frames

    @property
    def metadata(self) -> SourceMetadata:
        return self._meta

    @property
    def simulator(self) -> Simulator:
        return self._sim

    def frames(self):
        txs = self._meta.transmits
        period = len(txs) / self._meta.acquisition.prf
        vel = np.asarray(self._phantom.velocities, np.float64)
        moving = bool(np.any(vel != 0.0))
        pos0 = np.asarray(self._phantom.positions, np.float64) if moving else None
        i = 0
        while self._n_frames is None or i < self._n_frames:
            ph = self._phantom
            if moving and i > 0:
                ph = Phantom()
                ph.extend(self._phantom)
                ph.positions = (pos0 + vel * (i * period)).astype(np.float32)
            yield self._sim.simulate(txs, ph)
            i += 1


def _transmits_from_arrays(types, angles, focus, origin, delays, apod) -> list:
    out = []
    for e in range(len(types)):
        t = Transmit()
        t.type = _TX_TYPES[int(types[e])]
        t.angle = float(angles[e])
        t.focus = Vec3(*(float(v) for v in focus[e]))
        t.origin = Vec3(*(float(v) for v in origin[e]))
        t.delays = [float(v) for v in delays[e]]
        t.apodization = [float(v) for v in apod[e]]
        out.append(t)
    return out


class FileSource(RawSource):
    """Frames replayed from a `save_npz` recording (reference ingest.py:111-168).

    The RF array holds (frames x events, channels, samples); each frame is one
    block of `events_per_frame` events. `loop=True` replays without end.
    """

    def __init__(self, path, loop: bool = False):
        self.path = Path(path)
        self._loop = loop
        with np.load(self.path, allow_pickle=False) as z:
            self._rf = np.asarray(z["rf"], dtype=np.float32)
            probe = Probe()
            probe.n_elements = int(z["probe_n_elements"])
            probe.pitch = float(z["probe_pitch"])
            probe.element_width = float(z["probe_element_width"])
            probe.elevation_height = float(z["probe_elevation_height"])
            probe.center_frequency = float(z["probe_center_frequency"])
            probe.bandwidth = float(z["probe_bandwidth"])
            medium = Medium()
            medium.speed_of_sound = float(z["medium_speed_of_sound"])
            medium.attenuation = float(z["medium_attenuation"])
            acq = Acquisition()
            acq.sampling_frequency = float(z["acq_sampling_frequency"])
            acq.n_samples = int(z["acq_n_samples"])
            acq.t0 = float(z["acq_t0"])
            acq.prf = float(z["acq_prf"])
            txs = _transmits_from_arrays(z["tx_type"], z["tx_angle"], z["tx_focus"], z["tx_origin"],
                                         z["tx_delays"], z["tx_apodization"])
        self._meta = SourceMetadata(probe, medium, acq, txs)

    @property
    def metadata(self) -> SourceMetadata:
        return self._meta

    def frames(self):
        n_ev = len(self._meta.transmits)
        n_frames = max(1, self._rf.shape[0] // n_ev) if self._rf.ndim == 3 else 1
        m = self._meta
        while True:
            for f in range(n_frames):
                yield ChannelData.from_rf(self._rf[f * n_ev:(f + 1) * n_ev], m.probe, m.medium, m.acquisition,
                                          m.transmits)
            if not self._loop:
                return


class ArraySource(RawSource):
    """In-memory RF blocks (events, channels, samples), one per frame: the
    adapter a scanner driver writes against (reference ingest.py:171-183)."""

    def __init__(self, arrays, probe: Probe, medium: Medium, acquisition: Acquisition, transmits: list):
        self._arrays = arrays
        self._meta = SourceMetadata(probe, medium, acquisition, list(transmits))

    @property
    def metadata(self) -> SourceMetadata:
        return self._meta

    def frames(self):
        m = self._meta
        for a in self._arrays:
            yield ChannelData.from_rf(np.asarray(a, dtype=np.float32), m.probe, m.medium, m.acquisition,
                                      m.transmits)


def save_npz(path, data: ChannelData) -> Path:
    """Write channel data with every parameter needed to interpret it (the
    reference's recording layout, ingest.py:201-233)."""
    path = Path(path)
    txs = list(data.transmits)
    code = {t: i for i, t in enumerate(_TX_TYPES)}
    np.savez_compressed(
        path,
        rf=np.asarray(data.rf, dtype=np.float32),
        probe_n_elements=data.probe.n_elements,
        probe_pitch=data.probe.pitch,
        probe_element_width=data.probe.element_width,
        probe_elevation_height=data.probe.elevation_height,
        probe_center_frequency=data.probe.center_frequency,
        probe_bandwidth=data.probe.bandwidth,
        medium_speed_of_sound=data.medium.speed_of_sound,
        medium_attenuation=data.medium.attenuation,
        acq_sampling_frequency=data.acq.sampling_frequency,
        acq_n_samples=data.acq.n_samples,
        acq_t0=data.acq.t0,
        acq_prf=data.acq.prf,
        tx_type=np.array([code[t.type] for t in txs], dtype=np.int32),
        tx_angle=np.array([t.angle for t in txs], dtype=np.float32),
        tx_focus=np.array([[t.focus.x, t.focus.y, t.focus.z] for t in txs], dtype=np.float32).reshape(-1, 3),
        tx_origin=np.array([[t.origin.x, t.origin.y, t.origin.z] for t in txs], dtype=np.float32).reshape(-1, 3),
        tx_delays=np.array([list(t.delays) for t in txs], dtype=np.float32),
        tx_apodization=np.array([list(t.apodization) for t in txs], dtype=np.float32),
    )
    return path


@dataclass
class DeviceFrame:
    """One frame resident on the GPU: `rf` is a (events, channels, samples)
    float32 device tensor, ready on the consumer's stream. Its slot is refilled
    once the consumer asks for the next frame, behind the work the consumer had
    enqueued on its stream by then: use it (or copy it) on that stream before
    asking for the next frame."""

    index: int
    rf: object
    metadata: SourceMetadata


class DeviceFeed:
    """Streams a RawSource's frames into device memory ahead of the consumer.

    `stream` is the consumer's CUDA stream: a torch stream, a `usx.capi.Context`
    (its stream) or None for torch's current stream. `depth` frames are in
    flight: when the consumer asks for frame i, the copy of frame i + depth - 1
    is issued on a side stream (pinned host staging buffer, then one
    asynchronous host-to-device copy), behind an event that the consumer's
    stream recorded after its work on the frame that last used the slot, and
    frame i is handed over behind the event of its own copy. Every frame of a
    feed has one shape. Needs a CUDA device: there is no host fallback.
    """

    def __init__(self, source: RawSource, depth: int = 2, stream=None, device: int | None = None):
        import torch

        if not torch.cuda.is_available():
            raise RuntimeError("DeviceFeed: no CUDA device (this engine has no CPU path)")
        if depth < 1:
            raise ValueError("DeviceFeed: depth must be at least 1")
        self._torch = torch
        self._source = source
        self._depth = depth
        self._device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        if stream is None:
            stream = torch.cuda.current_stream(self._device)
        elif hasattr(stream, "stream") and callable(stream.stream):
            stream = torch.cuda.ExternalStream(stream.stream(), device=self._device)
        self._consumer = stream
        self._copy = torch.cuda.Stream(device=self._device)
        self._shape = None
        self._host = []
        self._dev = []
        self._copied = []
        self._released = []

    def _alloc(self, shape):
        torch = self._torch
        self._shape = shape
        for _ in range(self._depth):
            self._host.append(torch.empty(shape, dtype=torch.float32, pin_memory=True))
            self._dev.append(torch.empty(shape, dtype=torch.float32, device=self._device))
            self._copied.append(torch.cuda.Event())
            self._released.append(torch.cuda.Event())

    def _issue(self, k: int, rf) -> None:
        a = np.asarray(rf, dtype=np.float32)
        if self._shape is None:
            self._alloc(a.shape)
        elif a.shape != self._shape:
            raise ValueError(f"DeviceFeed: frame {k} has shape {a.shape}, the feed carries {self._shape}")
        slot = k % self._depth
        if k >= self._depth:
            self._copied[slot].synchronize()           # the pinned slot's previous copy has read it
            self._copy.wait_event(self._released[slot])  # the consumer is done with the device slot
        np.copyto(self._host[slot].numpy(), a)
        with self._torch.cuda.stream(self._copy):
            self._dev[slot].copy_(self._host[slot], non_blocking=True)
            self._copied[slot].record(self._copy)
        # The slot was allocated on another stream: tell the caching allocator
        # that the copy stream writes it, so that it is not handed out again
        # while a copy is in flight if the feed is dropped early.
        self._dev[slot].record_stream(self._copy)

    def __iter__(self):
        frames = iter(self._source.frames())
        issued = 0
        done = False
        i = 0
        while True:
            if i > 0:
                self._released[(i - 1) % self._depth].record(self._consumer)
            while not done and issued < i + self._depth:
                try:
                    cd = next(frames)
                except StopIteration:
                    done = True
                    break
                self._issue(issued, cd.rf)
                issued += 1
            if i >= issued:
                return
            slot = i % self._depth
            self._consumer.wait_event(self._copied[slot])
            yield DeviceFrame(i, self._dev[slot], self._source.metadata)
            i += 1

    def close(self) -> None:
        self._source.close()
