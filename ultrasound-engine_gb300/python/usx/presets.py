"""Probe and acquisition presets (same operating points as the reference's
python/usx/presets.py, so configurations carry over unchanged)."""

from __future__ import annotations

import numpy as np

from ._usx import Acquisition, Medium, Probe


def _probe(n, pitch, width, elev, f0, bw) -> Probe:
    p = Probe()
    p.n_elements = n
    p.pitch = pitch
    p.element_width = width
    p.elevation_height = elev
    p.center_frequency = f0
    p.bandwidth = bw
    return p


def linear_5mhz() -> Probe:
    """General-purpose 5 MHz linear array."""
    return _probe(128, 300e-6, 270e-6, 5e-3, 5.0e6, 0.65)


def linear_high_freq() -> Probe:
    """10 MHz fine-pitch linear array."""
    return _probe(128, 150e-6, 135e-6, 3e-3, 10.0e6, 0.7)


def phased_3mhz() -> Probe:
    """3 MHz phased array with half-wavelength pitch."""
    return _probe(64, 250e-6, 220e-6, 12e-3, 3.0e6, 0.6)


def acquisition(probe: Probe, depth: float = 0.06, medium: Medium | None = None,
                samples_per_wavelength: float = 8.0, prf: float | None = None) -> Acquisition:
    """An acquisition whose record covers the round trip to `depth` plus the
    transmit delay spread and the pulse length; PRF as fast as the depth allows."""
    med = medium or Medium()
    c = med.speed_of_sound
    a = Acquisition()
    a.sampling_frequency = float(samples_per_wavelength * probe.center_frequency)
    round_trip = 2.0 * depth / c
    margin = probe.aperture_width() / c + 4.0 / probe.center_frequency
    a.n_samples = int(np.ceil((round_trip + margin) * a.sampling_frequency))
    a.prf = float(prf) if prf else float(0.95 * c / (2.0 * depth))
    a.t0 = 0.0
    return a


def plane_wave_sequence(sim, half_angle_deg: float = 9.0, n_angles: int = 11):
    """Symmetric steered plane waves over +/- half_angle_deg."""
    if n_angles <= 1:
        return sim.make_plane_waves([0.0])
    return sim.make_plane_waves(list(np.deg2rad(np.linspace(-half_angle_deg, half_angle_deg, n_angles))))


def focused_sequence(sim, probe: Probe, n_lines: int = 128, focal_depth: float = 0.03):
    """Line-by-line focused scan across 90% of the aperture."""
    half = 0.5 * probe.aperture_width() * 0.9
    return sim.make_focused_scan(n_lines, -half, half, focal_depth)
