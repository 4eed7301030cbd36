"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference compiled from its sources).

Everything except the simulator is bit-exact: the oracle restates the
reference's float arithmetic operation by operation. The simulator sums
scatterer contributions in thread order, as the reference does under OpenMP,
so it is compared at a relative L2 of 1e-6."""

from __future__ import annotations

import numpy as np
import pytest

from gold import BF_CASES, rel_l2, sim_setup, txset
from oracle import oracle as O


def test_pulse_and_lowpass(oracle, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    import ctypes as C
    cfg = O.sim_config()
    f = oracle.lib.orc_pulse_f32
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, O.f32p, O.f32p]
    n = f(C.byref(pr), C.byref(acq), C.byref(cfg), None, None)
    p = np.zeros(n, np.float32)
    half = C.c_float()
    f(C.byref(pr), C.byref(acq), C.byref(cfg), p.ctypes.data_as(O.f32p), C.byref(half))
    assert np.array_equal(p, g["pulse"])
    assert half.value == pytest.approx(float(g["pulse_half"]), rel=0, abs=0)


def test_simulate_matches_reference(oracle, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    cd = O.channel_desc(pr, med, acq, txset(g, "pw"))
    rf = oracle.simulate(cd, O.sim_config(noise_db=-60.0, noise_seed=7), g["scat"], noise_z=g["noise_z"])
    assert rel_l2(rf, g["rf"]) < 1e-6
    quiet = oracle.simulate(cd, O.sim_config(noise_db=-200.0, incident_trim_db=-30.0, enable_motion=0), g["scat"])
    assert rel_l2(quiet, g["rf_quiet"]) < 1e-6


def test_demodulate_bit_exact(oracle, golden):
    g = golden("sim")
    pr, med, acq = sim_setup(g)
    cd = O.channel_desc(pr, med, acq, txset(g, "pw"))
    iq = oracle.demodulate(cd, O.demod_config(), g["rf"])
    assert np.array_equal(iq.astype(np.complex64), g["iq"])
    iq2 = oracle.demodulate(cd, O.demod_config(decimation=2, filter_taps=21, cutoff_fraction=0.45), g["rf"])
    assert np.array_equal(iq2.astype(np.complex64), g["iq_dec2"])


@pytest.mark.parametrize("name", sorted(BF_CASES))
def test_beamform_bit_exact(oracle, golden, name):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    cd = O.channel_desc(pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    out = oracle.beamform(cd, g["iq"], g["pts"], len(g["ax0"]), len(g["ax1"]), O.bf_config(**BF_CASES[name]))
    assert np.array_equal(out.astype(np.complex64), g[f"bf_{name}"])


def test_beamform_other_geometries_bit_exact(oracle, golden):
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    n0, n1 = len(g["ax0"]), len(g["ax1"])
    cd = O.channel_desc(pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    ev = oracle.beamform(cd, g["iq"], g["pts"], n0, n1, O.bf_config(f_number=1.5), 1, 2)
    assert np.array_equal(ev.astype(np.complex64), g["bf_das_ev1"])
    cdr = O.channel_desc(pr, med, acq, txset(s, "pw"))
    rf = oracle.beamform(cdr, s["rf"], g["pts"], n0, n1, O.bf_config(f_number=1.5))
    assert np.array_equal(rf.astype(np.complex64), g["bf_rf"])
    cdf = O.channel_desc(pr, med, acq, txset(g, "foc"), is_iq=True, fdem=5e6)
    sel = oracle.beamform(cdf, g["foc_iq"], g["pts"], n0, n1, O.bf_config(f_number=1.5, compounding=2))
    assert np.array_equal(sel.astype(np.complex64), g["bf_foc_select"])
    cdd = O.channel_desc(pr, med, acq, txset(g, "div"), is_iq=True, fdem=5e6)
    sec = oracle.beamform(cdd, g["div_iq"], g["spts"], len(g["sax0"]), len(g["sax1"]), O.bf_config(f_number=1.5))
    assert np.array_equal(sec.astype(np.complex64), g["bf_div_sector"])


@pytest.mark.parametrize("key,wt,order", [("w0o1", 0, 1), ("w1o1", 1, 1), ("w1o2", 1, 2), ("w2o0", 2, 0)])
def test_doppler_bit_exact(oracle, golden, key, wt, order):
    g = golden("doppler")
    ens = g["ens"]
    assert np.array_equal(oracle.wall_filter(ens, wt, order).astype(np.complex64), g[f"wall_{key}"])
    v, p, var, valid, nyq = oracle.color_flow(ens, g["ax1"], 5e6, 5000.0, 1540.0,
                                              O.doppler_config(wall_filter=wt, polynomial_order=order))
    assert np.array_equal(v, g[f"cf_vel_{key}"]) and np.array_equal(p, g[f"cf_pow_{key}"])
    assert np.array_equal(var, g[f"cf_var_{key}"]) and np.array_equal(valid, g[f"cf_valid_{key}"])
    assert np.float32(nyq) == g[f"cf_nyq_{key}"]
    assert np.array_equal(oracle.power_doppler(ens, wt, order), g[f"pd_{key}"])


def test_displacement_and_strain_bit_exact(oracle, golden):
    g = golden("doppler")
    ax, corr = oracle.displacement(g["disp_a"], g["disp_b"], g["disp_ax1"], 5e6, 1540.0, 4, 1, 5)
    assert np.array_equal(ax, g["disp_axial"]) and np.array_equal(corr, g["disp_corr"])
    assert np.array_equal(oracle.strain(ax, g["disp_ax1"], 9), g["strain"])


def test_postprocess_bit_exact(oracle, golden):
    g = golden("post")
    b = golden("bf")
    assert np.array_equal(oracle.envelope(g["frame"], 5e6), g["env_iq"])
    assert np.array_equal(oracle.envelope(g["rf_frame"], 0.0), g["env_rf"])
    assert np.array_equal(oracle.apply_tgc(g["env_iq"], b["pts"], 0.5, 5e6), g["tgc"])
    assert np.array_equal(oracle.log_compress(g["tgc"], 50.0, 2.0, -1.0), g["log"])
    px, ext = oracle.scan_convert(g["sc_img"], 1, b["sax0"], b["sax1"], (0, 0, 0), b["spts"], 50, 40, -1.0)
    assert np.array_equal(px, g["sc_sector"]) and np.array_equal(ext, g["sc_sector_ext"])
    px, _ = oracle.scan_convert(g["env_iq"], 0, b["ax0"], b["ax1"], (0, 0, 0), b["pts"], 33, 47, 0.0)
    assert np.array_equal(px, g["sc_cart"])


def test_fp64_oracle_tracks_fp32(oracle, golden):
    """The double-precision build runs the same algorithm: FP32 DAS sits within
    the reference's own FP32 rounding (~3e-5 relative L2) of it."""
    g = golden("bf")
    s = golden("sim")
    pr, med, acq = sim_setup(s)
    cd = O.channel_desc(pr, med, acq, txset(s, "pw"), is_iq=True, fdem=5e6)
    f64 = oracle.beamform(cd, g["iq"], g["pts"], len(g["ax0"]), len(g["ax1"]), O.bf_config(f_number=1.5), prec="f64")
    assert rel_l2(g["bf_das"], f64) < 2e-4
