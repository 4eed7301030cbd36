"""Host-side logic without a GPU: seeded phantoms, delay laws, grids and the
metrics against the reference's own outputs, and the presets' sizing."""

from __future__ import annotations

import numpy as np
import pytest

import usx
from gold import sim_setup


def test_speckle_box_draws_like_the_reference(golden):
    g = golden("sim")
    ph = usx.Phantom.speckle_box(-0.006, 0.006, 0.006, 0.022, 0.0, 600, 11)
    ph.scale_amplitude_in_circle(usx.Vec3(0.0, 0.0, 0.014), 0.002, 0.0)
    ref = g["scat"][:600]
    assert np.array_equal(np.asarray(ph.positions), ref[:, :3])
    assert np.array_equal(np.asarray(ph.amplitudes), ref[:, 3])


def test_flow_tube_draws_like_the_reference(golden):
    g = golden("sim")
    ph = usx.Phantom()
    ph.add_flow_tube(usx.Vec3(0.001, 0.0, 0.016), 0.0015, 0.01, 0.4, 0.3, 40, 5, 0.5)
    ref = g["scat"][602:]
    assert np.array_equal(np.asarray(ph.positions), ref[:, :3])
    assert np.array_equal(np.asarray(ph.amplitudes), ref[:, 3])
    assert np.array_equal(np.asarray(ph.velocities), ref[:, 4:7])


def test_plane_wave_delays_match_the_reference(golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = pr.n_elements, pr.pitch, pr.element_width
    probe.center_frequency, probe.bandwidth = pr.center_frequency, pr.bandwidth
    a = usx.Acquisition()
    a.sampling_frequency, a.n_samples, a.prf = acq.sampling_frequency, acq.n_samples, acq.prf
    sim = usx.Simulator(probe, usx.Medium(), a)
    txs = sim.make_plane_waves([float(x) for x in g["pw_angles"]])
    for e, t in enumerate(txs):
        assert np.array_equal(np.asarray(t.delays, np.float32), g["pw_delays"][e])
        assert np.array_equal(np.asarray(t.apodization, np.float32), g["pw_apod"][e])
    assert np.array_equal(np.asarray(sim.pulse()), g["pulse"])


def test_focused_and_diverging_delays_match_the_reference(golden):
    g = golden("bf")
    s = golden("sim")
    pr, _, _ = sim_setup(s)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = pr.n_elements, pr.pitch, pr.element_width
    for prefix in ("foc", "div"):
        for e in range(len(g[f"{prefix}_types"])):
            t = usx.Transmit()
            t.type = usx.TransmitType.FOCUSED if prefix == "foc" else usx.TransmitType.DIVERGING
            t.angle = float(g[f"{prefix}_angles"][e])
            t.focus = usx.Vec3(*[float(v) for v in g[f"{prefix}_focus"][e]])
            t.origin = usx.Vec3(*[float(v) for v in g[f"{prefix}_origin"][e]])
            usx.compute_transmit_delays(probe, usx.Medium(), t)
            assert np.array_equal(np.asarray(t.delays, np.float32), g[f"{prefix}_delays"][e])
            assert np.array_equal(np.asarray(t.apodization, np.float32), g[f"{prefix}_apod"][e])


def test_grids_match_the_reference(golden):
    g = golden("bf")
    cart = usx.ScanGrid.cartesian(-0.006, 0.006, 16, 0.006, 0.022, 40)
    assert np.array_equal(np.asarray(cart.points), g["pts"])
    sec = usx.ScanGrid.sector(-0.5, 0.5, 20, 0.006, 0.022, 36, usx.Vec3(0, 0, 0))
    assert np.array_equal(np.asarray(sec.points), g["spts"])
    assert sec.shape == (20, 36) and cart.n_pixels == 640


def test_acquisition_preset_covers_the_depth():
    p = usx.presets.linear_5mhz()
    for depth in (0.03, 0.06, 0.12):
        a = usx.presets.acquisition(p, depth=depth)
        assert a.n_samples / a.sampling_frequency >= 2 * depth / 1540.0
        assert a.max_depth(1540.0) >= depth
    # the 20 MHz, 50 mm record of the 11-plane-wave workload is 1814 samples
    a = usx.presets.acquisition(p, depth=0.05, samples_per_wavelength=4.0)
    assert a.n_samples == int(np.ceil((2 * 0.05 / 1540 + p.aperture_width() / 1540 + 4 / 5e6) * 20e6))


def test_probe_geometry():
    p = usx.presets.linear_5mhz()
    x = np.asarray(p.element_x)
    assert len(x) == p.n_elements
    assert np.allclose(x.mean(), 0.0, atol=1e-9)
    assert np.allclose(np.diff(x), p.pitch, rtol=1e-5)
    assert usx.presets.phased_3mhz().pitch < 0.55 * usx.presets.phased_3mhz().wavelength(1540)


def test_gcnr_is_invariant_to_monotone_transforms():
    grid = usx.ScanGrid.cartesian(-0.008, 0.008, 60, 0.018, 0.032, 120)
    rng = np.random.default_rng(0)
    x = np.asarray(grid.axis0)[:, None]
    z = np.asarray(grid.axis1)[None, :]
    inside = np.hypot(x, z - 0.025) < 0.003
    env = np.abs(rng.normal(size=(60, 120)) + 1j * rng.normal(size=(60, 120)))
    env = np.where(inside, env * 0.15, env)
    g1 = usx.metrics.gcnr(env, grid, (0.0, 0.025), 0.003)
    assert g1 == pytest.approx(usx.metrics.gcnr(np.sqrt(env), grid, (0.0, 0.025), 0.003), abs=1e-12)
    assert g1 == pytest.approx(usx.metrics.gcnr(env ** 2.5, grid, (0.0, 0.025), 0.003), abs=1e-12)
    assert 0.2 < g1 <= 1.0
    c1 = usx.metrics.cnr(env, grid, (0.0, 0.025), 0.003)
    assert abs(c1 - usx.metrics.cnr(env ** 2.5, grid, (0.0, 0.025), 0.003)) > 0.05 * c1


def test_metrics_match_reference_values(golden):
    g = golden("metrics")
    env = g["env"]
    grid = usx.ScanGrid.cartesian(float(g["grid"][0]), float(g["grid"][1]), int(g["grid"][2]),
                                  float(g["grid"][3]), float(g["grid"][4]), int(g["grid"][5]))
    s = usx.metrics.summarize(env, grid, lesion_xz=(0.0, 0.014), lesion_radius=0.002, wire_xz=(-0.003, 0.010),
                              speckle_xz=(0.003, 0.018), speckle_half=(0.002, 0.002))
    for k, v in zip(g["keys"], g["values"]):
        assert s[str(k)] == pytest.approx(float(v), rel=1e-12, abs=1e-12, nan_ok=True), k
