"""usx — the usx ultrasound imaging path on NVIDIA GB300.

Drop-in for the reference package's Python surface (python/usx/__init__.py of
AadithyaSairam/ultrasound-engine): the same classes and functions, re-exported
from the `_usx` extension, whose compute runs as CUDA kernels for sm_103a.
There is no CPU path: without a usable GPU, compute calls raise RuntimeError.

    import usx
    probe = usx.presets.linear_5mhz()
    sim   = usx.Simulator(probe, usx.Medium(), usx.presets.acquisition(probe))
    raw   = sim.simulate(sim.make_plane_waves(usx.angles_deg(-9, 9, 11)),
                         usx.phantoms.cyst_phantom(probe))
    frame = usx.ImagingPipeline(usx.grid_for(probe)).process_frame(raw)
    bmode = usx.to_bmode(frame)
"""

from __future__ import annotations

import numpy as np

from ._usx import (  # noqa: F401
    Acquisition,
    Beamformer,
    BeamformerConfig,
    ChannelData,
    ColorFlowMap,
    Combiner,
    Compounding,
    DemodConfig,
    DisplacementMap,
    DopplerConfig,
    Frame,
    GridType,
    ImagingPipeline,
    Medium,
    MvSolver,
    Phantom,
    PipelineConfig,
    PipelineStats,
    Probe,
    ScanConverted,
    ScanGrid,
    Scatterer,
    SimulatorConfig,
    Simulator,
    Transmit,
    TransmitType,
    Vec3,
    WallFilter,
    Window,
    apply_tgc,
    apply_wall_filter,
    axial_strain,
    color_flow,
    compute_transmit_delays,
    demodulate,
    design_lowpass,
    element_directivity,
    envelope,
    estimate_axial_displacement,
    log_compress,
    power_doppler,
    scan_convert,
    transmit_arrival_time,
    transmit_sensitivity,
    window_value,
    __version__,
    __backend__,
)

from . import ingest, metrics, phantoms, presets  # noqa: E402,F401

__all__ = [n for n in dir() if not n.startswith("_")] + [
    "angles_deg", "to_bmode", "grid_for", "extent_mm",
]


def angles_deg(start: float, stop: float, count: int) -> list[float]:
    """Evenly spaced steering angles given in degrees, returned in radians."""
    if count == 1:
        return [np.deg2rad(0.5 * (start + stop))]
    return list(np.deg2rad(np.linspace(start, stop, count)))


def to_bmode(frame: Frame, dynamic_range_db: float = 60.0, gain_db: float = 0.0,
             medium: Medium | None = None, tgc: bool = True) -> np.ndarray:
    """Complex frame to a log-compressed image in [0, 1], shaped (axis0, axis1)."""
    env = envelope(frame)
    if tgc:
        med = medium or Medium()
        f0 = frame.demodulation_frequency or 5.0e6
        env = apply_tgc(env, frame.grid, med.attenuation, f0)
    return log_compress(env, dynamic_range_db, gain_db, -1.0)


def grid_for(probe: Probe, z_min: float = 0.005, z_max: float = 0.055,
             n_lateral: int = 256, n_axial: int = 768,
             width: float | None = None) -> ScanGrid:
    """A Cartesian grid spanning the probe's aperture (or `width`) over a depth range."""
    half = 0.5 * (width if width is not None else probe.aperture_width())
    return ScanGrid.cartesian(-half, half, n_lateral, z_min, z_max, n_axial)


def extent_mm(grid: ScanGrid) -> tuple[float, float, float, float]:
    """Display extent in millimetres (left, right, bottom, top) for an (axis0, axis1) image."""
    a0 = np.asarray(grid.axis0) * 1e3
    a1 = np.asarray(grid.axis1) * 1e3
    return (float(a0[0]), float(a0[-1]), float(a1[-1]), float(a1[0]))
