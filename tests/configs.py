"""The five benchmark configurations as test inputs.

Each builder returns host objects made by this engine's `usx` host code
(probe, medium, acquisition, transmits, grid, phantom), whose seeded phantom
factories and delay laws are pinned to the reference's by tests/test_host.py,
plus the matching oracle descriptors. The same phantom and transmit tables
feed both the GPU path and the oracle, so seeded inputs are never regenerated
on the device.

Sizes and fixed choices (the configurations leave these open):
  cfg1  128 el, 5 MHz, pitch 0.3 mm, width 0.27 mm, 60% bandwidth; fs 20 MHz,
        depth 50 mm (1814 samples); 11 plane waves at -9..9 deg; 20,000
        scatterers uniform in x in [-19, 19] mm, z in [5, 50] mm, N(0,1)
        amplitudes, an anechoic 3 mm cyst at (0, 20 mm) whose scatterers get
        zero amplitude (an exact zero contribution, the same RF as removing
        them), five wires of amplitude 20 at x = -12 mm, z = 10..50 mm;
        256 x 640 grid over the aperture and z = 5-50 mm.
  cfg2  the same probe, 75 plane waves at -16..16 deg, depth 60 mm (2073
        samples), 100,000 scatterers with cysts of radius 2, 3 and 4 mm,
        512 x 1024 grid over the aperture and z = 5-60 mm.
  cfg4  Doppler: 3 mm vessel at 25 deg, parabolic flow, 0.4 m/s peak, blood
        at 0.1 x the tissue amplitude, tissue drifting axially at 5 mm/s,
        3 plane waves at -5..5 deg per pulse, PRF 5 kHz, 256 x 512 grid over
        z = 10-35 mm. Strain: a 4 x stiff 5 mm inclusion at 30 mm under 1%
        compression, one plane wave, 256 x 1024 grid over z = 12-48 mm.
  cfg5  phased array: 64 el, 2.5 MHz, pitch 0.2 mm, width 0.18 mm, 31
        diverging waves over +/-45 deg with the virtual source 10 mm behind
        the array, 256 beams x 1024 samples to 80 mm, scan conversion to
        800 x 800.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from oracle import oracle as O


@dataclass
class Setup:
    usx: object
    probe: object
    medium: object
    acq: object
    sim: object
    txs: list
    grid: object
    phantom: object = None


def linear_probe(usx, n=128, pitch=300e-6, width=270e-6, f0=5e6, bw=0.6):
    p = usx.Probe()
    p.n_elements, p.pitch, p.element_width = n, pitch, width
    p.center_frequency, p.bandwidth = f0, bw
    return p


def scatterers(ph) -> np.ndarray:
    """Phantom -> the C-ABI's 8-float scatterer rows (position, amplitude, velocity)."""
    pos, amp, vel = np.asarray(ph.positions), np.asarray(ph.amplitudes), np.asarray(ph.velocities)
    sc = np.zeros((len(amp), 8), np.float32)
    sc[:, :3], sc[:, 3], sc[:, 4:7] = pos, amp, vel
    return sc


def o_probe(p):
    return O.probe(n_elements=p.n_elements, pitch=p.pitch, element_width=p.element_width,
                   elevation_height=p.elevation_height, center_frequency=p.center_frequency,
                   bandwidth=p.bandwidth)


def o_medium(m):
    return O.medium(m.speed_of_sound, m.attenuation, m.density)


def o_acq(a):
    return O.acquisition(fs=a.sampling_frequency, n_samples=a.n_samples, t0=a.t0, prf=a.prf)


def o_txset(txs) -> O.TxSet:
    n = len(txs)
    return O.TxSet(np.asarray([int(t.type.value) for t in txs], np.int32),
                   np.asarray([t.angle for t in txs], np.float32),
                   np.asarray([(t.focus.x, t.focus.y, t.focus.z) for t in txs], np.float32).reshape(n, 3),
                   np.asarray([(t.origin.x, t.origin.y, t.origin.z) for t in txs], np.float32).reshape(n, 3),
                   np.asarray([t.delays for t in txs], np.float32),
                   np.asarray([t.apodization for t in txs], np.float32))


def o_channel(s: Setup, is_iq=False, fdem=0.0, txs=None):
    return O.channel_desc(o_probe(s.probe), o_medium(s.medium), o_acq(s.acq), o_txset(txs or s.txs),
                          is_iq=is_iq, fdem=fdem)


def capi_channel(capi, s: Setup, is_iq=False, fdem=0.0, txs=None):
    t = o_txset(txs or s.txs)
    tx = [dict(type=int(t.types[e]), angle=float(t.angles[e]), focus=t.focus[e], origin=t.origin[e],
               delays=t.delays[e], apodization=t.apod[e]) for e in range(len(t))]
    p, m, a = s.probe, s.medium, s.acq
    return capi.Channel(capi.Probe(p.n_elements, p.pitch, p.element_width, p.elevation_height,
                                   p.center_frequency, p.bandwidth),
                        capi.Medium(m.speed_of_sound, m.attenuation, m.density),
                        capi.Acquisition(a.sampling_frequency, a.n_samples, a.t0, a.prf), tx, is_iq, fdem)


def capi_grid(capi, grid, gtype=0):
    return capi.Grid(gtype, np.asarray(grid.axis0), np.asarray(grid.axis1),
                     np.asarray(grid.points, np.float32).reshape(-1, 3))


CFG1_CYST = (0.0, 0.020, 0.003)
CFG1_WIRES = tuple((-0.012, z) for z in (0.010, 0.020, 0.030, 0.040, 0.050))


def cfg1(seed: int = 11) -> Setup:
    import usx
    probe = linear_probe(usx)
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.050, medium=medium, samples_per_wavelength=4.0)
    assert acq.n_samples == 1814
    scfg = usx.SimulatorConfig()
    scfg.noise_db = -200.0
    sim = usx.Simulator(probe, medium, acq, scfg)
    txs = sim.make_plane_waves(usx.angles_deg(-9, 9, 11))
    ph = usx.Phantom.speckle_box(-0.019, 0.019, 0.005, 0.050, 0.0, 20_000, seed)
    ph.scale_amplitude_in_circle(usx.Vec3(CFG1_CYST[0], 0.0, CFG1_CYST[1]), CFG1_CYST[2], 0.0)
    ph.extend(usx.Phantom.point_targets([usx.Vec3(x, 0.0, z) for x, z in CFG1_WIRES], 20.0))
    grid = usx.grid_for(probe, 0.005, 0.050, 256, 640)
    return Setup(usx, probe, medium, acq, sim, txs, grid, ph)


CFG2_CYSTS = ((-0.010, 0.025, 0.002), (0.0, 0.035, 0.003), (0.010, 0.045, 0.004))


def cfg2(seed: int = 2026, n_scat: int = 100_000) -> Setup:
    import usx
    probe = linear_probe(usx)
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.060, medium=medium, samples_per_wavelength=4.0)
    assert acq.n_samples == 2073
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    txs = sim.make_plane_waves(usx.angles_deg(-16, 16, 75))
    half = 0.5 * probe.aperture_width()
    ph = usx.Phantom.speckle_box(-half * 1.1, half * 1.1, 0.004, 0.062, 0.0, n_scat, seed)
    for x, z, r in CFG2_CYSTS:
        ph.scale_amplitude_in_circle(usx.Vec3(x, 0.0, z), r, 0.0)
    grid = usx.grid_for(probe, 0.005, 0.060, 512, 1024)
    return Setup(usx, probe, medium, acq, sim, txs, grid, ph)


def cfg4_doppler(n_pulses: int = 32) -> Setup:
    import usx
    probe = linear_probe(usx)
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.04, medium=medium, samples_per_wavelength=4.0)
    acq.prf = 5000.0
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    txs = sim.make_plane_waves(usx.angles_deg(-5, 5, 3) * n_pulses)
    ph = usx.phantoms.flow_phantom(probe, medium, vessel_depth=0.022, vessel_radius=0.003, angle_deg=25.0,
                                  peak_velocity=0.4, z_min=0.005, z_max=0.04)
    grid = usx.grid_for(probe, 0.01, 0.035, 256, 512)
    return Setup(usx, probe, medium, acq, sim, txs, grid, ph)


def cfg4_doppler_scatterers(ph) -> np.ndarray:
    """Blood at 0.1 x the tissue's mean |amplitude|, tissue drifting at 5 mm/s."""
    sc = scatterers(ph)
    blood = np.linalg.norm(sc[:, 4:7], axis=1) > 0
    ratio = np.abs(sc[blood, 3]).mean() / max(1e-12, np.abs(sc[~blood, 3]).mean())
    sc[blood, 3] *= np.float32(0.1 / max(1e-12, ratio))
    sc[~blood, 6] = 0.005
    return sc


def cfg4_strain() -> tuple[Setup, list]:
    import usx
    probe = linear_probe(usx)
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.05, medium=medium, samples_per_wavelength=4.0)
    scfg = usx.SimulatorConfig()
    scfg.noise_db = -200.0
    scfg.enable_motion = False
    sim = usx.Simulator(probe, medium, acq, scfg)
    txs = sim.make_plane_waves(usx.angles_deg(0, 0, 1))
    grid = usx.grid_for(probe, 0.012, 0.048, 256, 1024)
    phs = [usx.phantoms.elastography_phantom(probe, medium, strain=s) for s in (0.0, 0.01)]
    return Setup(usx, probe, medium, acq, sim, txs, grid), phs


def cfg5_sector(n_scat: int = 100_000) -> Setup:
    import usx
    probe = linear_probe(usx, n=64, pitch=200e-6, width=180e-6, f0=2.5e6)
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.082, medium=medium, samples_per_wavelength=4.0)
    scfg = usx.SimulatorConfig()
    scfg.noise_db = -200.0
    sim = usx.Simulator(probe, medium, acq, scfg)
    txs = sim.make_diverging_waves(usx.angles_deg(-45, 45, 31), 0.01)
    ph = usx.Phantom.speckle_box(-0.06, 0.06, 0.004, 0.084, 0.0, n_scat, 2027)
    for x, z, r in ((-0.015, 0.04, 0.004), (0.02, 0.06, 0.005)):
        ph.scale_amplitude_in_circle(usx.Vec3(x, 0.0, z), r, 0.0)
    grid = usx.ScanGrid.sector(float(np.deg2rad(-45.0)), float(np.deg2rad(45.0)), 256, 0.005, 0.08, 1024,
                               usx.Vec3(0.0, 0.0, 0.0))
    return Setup(usx, probe, medium, acq, sim, txs, grid, ph)


def image_metrics(env, grid, cyst, wires, speckle_xz) -> dict:
    """The reference's image-quality numbers (python/usx/metrics.py) of one frame."""
    from usx import metrics as M
    out = {"cnr": M.cnr(env, grid, cyst[:2], cyst[2]), "gcnr": M.gcnr(env, grid, cyst[:2], cyst[2]),
           "speckle_snr": M.speckle_snr(env, grid, speckle_xz, (0.004, 0.004))}
    for k, w in enumerate(wires):
        psf = M.measure_psf(env, grid, w)
        out[f"wire{k}_lateral_fwhm"] = psf.lateral_fwhm
        out[f"wire{k}_axial_fwhm"] = psf.axial_fwhm
    return out
