"""Standard test phantoms: wires (resolution), cysts (contrast), a flow tube
(Doppler) and a stiff inclusion (elastography). Same targets, seeds and
scatterer densities as the reference's python/usx/phantoms.py, so a phantom
named here is the same phantom there."""

from __future__ import annotations

import numpy as np

from ._usx import Medium, Phantom, Probe, Vec3


def _speckle(probe: Probe, medium: Medium, x_half: float, z_min: float, z_max: float,
             y_half: float, seed: int, density_per_cell: float) -> Phantom:
    n = Phantom.recommended_scatterer_count(probe, medium, 2 * x_half, z_max - z_min, 2 * y_half,
                                            f_number=2.0, per_cell=density_per_cell)
    n = int(min(max(n, 2000), 400_000))
    return Phantom.speckle_box(-x_half, x_half, z_min, z_max, y_half, n, seed)


def wire_targets(depths=(0.010, 0.020, 0.030, 0.040, 0.050), lateral=(-0.006, 0.0, 0.006)) -> Phantom:
    """A grid of isolated point scatterers (the point spread function)."""
    return Phantom.point_targets([Vec3(float(x), 0.0, float(z)) for z in depths for x in lateral], 1.0)


def cyst_phantom(probe: Probe, medium: Medium | None = None,
                 cysts=((0.0, 0.020, 0.003, 0.0), (-0.007, 0.035, 0.003, 0.25), (0.007, 0.035, 0.003, 2.5)),
                 z_min: float = 0.005, z_max: float = 0.055, seed: int = 3,
                 density_per_cell: float = 12.0) -> Phantom:
    """Speckle background with inclusions given as (x, z, radius, amplitude scale)."""
    med = medium or Medium()
    half = 0.5 * probe.aperture_width() * 1.15
    ph = _speckle(probe, med, half, z_min, z_max, 2e-4, seed, density_per_cell)
    for x, z, r, scale in cysts:
        ph.scale_amplitude_in_circle(Vec3(float(x), 0.0, float(z)), float(r), float(scale))
    return ph


def resolution_and_contrast(probe: Probe, medium: Medium | None = None, z_min: float = 0.005,
                            z_max: float = 0.055, seed: int = 5) -> Phantom:
    """Wires for resolution plus an anechoic cyst for contrast."""
    ph = cyst_phantom(probe, medium, cysts=((0.006, 0.030, 0.0035, 0.0),), z_min=z_min, z_max=z_max, seed=seed)
    ph.extend(Phantom.point_targets([Vec3(-0.008, 0.0, float(z)) for z in (0.012, 0.024, 0.036, 0.048)], 40.0))
    return ph


def flow_phantom(probe: Probe, medium: Medium | None = None, vessel_depth: float = 0.025,
                 vessel_radius: float = 0.004, angle_deg: float = 20.0, peak_velocity: float = 0.35,
                 z_min: float = 0.005, z_max: float = 0.045, seed: int = 7,
                 with_tissue: bool = True) -> Phantom:
    """A vessel with laminar flow inside stationary tissue."""
    med = medium or Medium()
    ph = Phantom()
    if with_tissue:
        half = 0.5 * probe.aperture_width() * 1.15
        ph = _speckle(probe, med, half, z_min, z_max, 2e-4, seed, 10.0)
        ph.scale_amplitude_in_circle(Vec3(0.0, 0.0, vessel_depth), vessel_radius, 0.0)
    ph.add_flow_tube(Vec3(0.0, 0.0, vessel_depth), vessel_radius, 0.06, float(np.deg2rad(angle_deg)),
                     peak_velocity, 20000, seed + 1, 0.03)
    return ph


def elastography_phantom(probe: Probe, medium: Medium | None = None, inclusion=(0.0, 0.030, 0.005),
                         stiffness_ratio: float = 4.0, strain: float = 0.0, z_min: float = 0.010,
                         z_max: float = 0.050, seed: int = 13) -> Phantom:
    """Soft background with a stiff inclusion, compressed by a bulk axial `strain`.

    The displacement at depth z integrates the local strain down the line, the
    strain being divided by `stiffness_ratio` over the chord of the inclusion
    crossed, so the displacement field is continuous."""
    med = medium or Medium()
    half = 0.5 * probe.aperture_width() * 1.15
    ph = _speckle(probe, med, half, z_min, z_max, 2e-4, seed, 12.0)
    if strain == 0.0:
        return ph
    cx, cz, r = inclusion
    pos = np.asarray(ph.positions, dtype=np.float64)
    x, z = pos[:, 0], pos[:, 2]
    chord = 2.0 * np.sqrt(np.clip(r * r - (x - cx) ** 2, 0.0, None))
    crossed = np.clip(z - (cz - 0.5 * chord), 0.0, chord)
    e_soft = float(strain)
    e_stiff = e_soft / float(stiffness_ratio)
    moved = pos.copy()
    moved[:, 2] = z + e_soft * (z - z_min) + (e_stiff - e_soft) * crossed
    out = ph.copy()
    out.positions = moved.astype(np.float32)
    out.amplitudes = np.asarray(ph.amplitudes, dtype=np.float32)
    return out
