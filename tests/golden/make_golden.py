"""Generate the golden fixtures in this directory from the reference engine.

Runs the reference (AadithyaSairam/ultrasound-engine) compiled from its own
sources by oracle/build_ref.sh into oracle/_ref/libusx_ref.so, on small seeded
inputs, and stores inputs and outputs as compressed npz files. The fixtures
pin both the CPU oracle (tests/test_oracle_golden.py) and the CUDA kernels
(tests/test_gpu_parity.py) to the reference's own results.

    python oracle/build_ref.sh && python tests/golden/make_golden.py
"""

from __future__ import annotations

import sys
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))

from oracle import oracle as O  # noqa: E402

# The reference checkout: $USX_REFERENCE_DIR, else where this container mounts it.
REF_DIR = Path(os.environ.get("USX_REFERENCE_DIR", "/root/reference"))


def tx_arrays(txs: O.TxSet, prefix: str) -> dict:
    return {f"{prefix}_types": txs.types, f"{prefix}_angles": txs.angles, f"{prefix}_focus": txs.focus,
            f"{prefix}_origin": txs.origin, f"{prefix}_delays": txs.delays, f"{prefix}_apod": txs.apod}


def main() -> None:
    ref = O.RefLib()
    rng = np.random.default_rng(20261203)

    # ---- simulation + demodulation: 32-element linear probe, 3 plane waves ----
    pr = O.probe(n_elements=32, pitch=300e-6, element_width=270e-6, center_frequency=5e6, bandwidth=0.6)
    med = O.medium()
    acq = O.acquisition(fs=20e6, n_samples=640, prf=5000.0)
    angles = np.deg2rad(np.linspace(-9, 9, 3)).astype(np.float32)
    txs = ref.transmits(pr, med, "plane", angles)
    scat = ref.speckle_box(-0.006, 0.006, 0.006, 0.022, 0.0, 600, seed=11)
    scat = ref.scale_in_circle(scat, 0.0, 0.014, 0.002, 0.0)
    wires = np.zeros((2, 8), np.float32)
    wires[:, 0] = [-0.003, 0.002]
    wires[:, 2] = [0.010, 0.018]
    wires[:, 3] = 20.0
    moving = ref.flow_tube(0.001, 0.016, 0.0015, 0.01, 0.4, 0.3, 40, seed=5, amplitude=0.5)
    scat = np.concatenate([scat, wires, moving])
    cd = O.channel_desc(pr, med, acq, txs)
    scfg = O.sim_config(noise_db=-60.0, noise_seed=7)
    rf = ref.simulate(cd, scfg, scat)
    ev_size = pr.n_elements * acq.n_samples
    noise_z = np.concatenate([ref.normals(7 + e, ev_size) for e in range(len(txs))])
    scfg_quiet = O.sim_config(noise_db=-200.0, incident_trim_db=-30.0, enable_motion=0)
    rf_quiet = ref.simulate(cd, scfg_quiet, scat)
    pulse, pulse_half = ref.pulse(cd, scfg)
    iq = ref.demodulate(cd, O.demod_config(), rf)
    iq_dec2 = ref.demodulate(cd, O.demod_config(decimation=2, filter_taps=21, cutoff_fraction=0.45), rf)
    np.savez_compressed(
        HERE / "golden_sim.npz", scat=scat, rf=rf, rf_quiet=rf_quiet, noise_z=noise_z, pulse=pulse,
        pulse_half=np.float32(pulse_half), iq=iq, iq_dec2=iq_dec2, **tx_arrays(txs, "pw"),
        probe=np.array([pr.n_elements, pr.pitch, pr.element_width, pr.center_frequency, pr.bandwidth], np.float64),
        acq=np.array([acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf], np.float64))

    # ---- beamforming on that IQ ------------------------------------------------
    ax0, ax1, pts = ref.grid(0, -0.006, 0.006, 16, 0.006, 0.022, 40)
    cdq = O.channel_desc(pr, med, acq, txs, is_iq=True, fdem=5e6)
    out = {"ax0": ax0, "ax1": ax1, "pts": pts, "iq": iq}
    cases = {
        "das": dict(f_number=1.5),
        "das_rect": dict(f_number=1.0, rx_window=0, transmit_weighting=0),
        "das_tukey": dict(f_number=1.2, rx_window=3, tukey_alpha=0.3),
        "cf": dict(f_number=1.5, coherence_factor=1),
        "dmas": dict(f_number=1.5, combiner=1),
        "mv": dict(f_number=1.5, combiner=2, mv_subarray=16, mv_range_average=2),
        "mv_l4": dict(f_number=2.5, combiner=2, mv_subarray=4, mv_range_average=1, mv_diagonal_loading=0.05),
        "mv_cf": dict(f_number=1.5, combiner=2, mv_subarray=8, coherence_factor=1),
        "incoh": dict(f_number=1.5, compounding=1),
        "select": dict(f_number=1.5, compounding=2),
        "dmas_incoh": dict(f_number=1.5, combiner=1, compounding=1),
    }
    for name, kw in cases.items():
        out[f"bf_{name}"] = ref.beamform(cdq, iq, 0, ax0, ax1, (0, 0, 0), pts, O.bf_config(**kw))
    out["bf_das_ev1"] = ref.beamform(cdq, iq, 0, ax0, ax1, (0, 0, 0), pts, O.bf_config(f_number=1.5), 1, 2)
    # RF beamforming (no demodulation).
    cdr = O.channel_desc(pr, med, acq, txs)
    out["bf_rf"] = ref.beamform(cdr, rf, 0, ax0, ax1, (0, 0, 0), pts, O.bf_config(f_number=1.5))
    # Focused transmits with Select compounding, diverging waves on a sector grid.
    ftx = ref.transmits(pr, med, "focused", [(x, 0.014, 0.0) for x in np.linspace(-0.004, 0.004, 5)])
    cdf = O.channel_desc(pr, med, acq, ftx)
    rf_f = ref.simulate(cdf, scfg_quiet, scat)
    iq_f = ref.demodulate(cdf, O.demod_config(), rf_f)
    cdfq = O.channel_desc(pr, med, acq, ftx, is_iq=True, fdem=5e6)
    out["foc_iq"] = iq_f
    out.update(tx_arrays(ftx, "foc"))
    out["bf_foc_select"] = ref.beamform(cdfq, iq_f, 0, ax0, ax1, (0, 0, 0), pts,
                                        O.bf_config(f_number=1.5, compounding=2))
    out["bf_foc_coh"] = ref.beamform(cdfq, iq_f, 0, ax0, ax1, (0, 0, 0), pts, O.bf_config(f_number=1.5))
    dtx = ref.transmits(pr, med, "diverging", [(a, 0.01) for a in np.deg2rad([-20.0, 0.0, 20.0])])
    cdd = O.channel_desc(pr, med, acq, dtx)
    rf_d = ref.simulate(cdd, scfg_quiet, scat)
    iq_d = ref.demodulate(cdd, O.demod_config(), rf_d)
    cddq = O.channel_desc(pr, med, acq, dtx, is_iq=True, fdem=5e6)
    sx0, sx1, spts = ref.grid(1, -0.5, 0.5, 20, 0.006, 0.022, 36, apex=(0.0, 0.0, 0.0))
    out.update(tx_arrays(dtx, "div"))
    out.update(div_iq=iq_d, sax0=sx0, sax1=sx1, spts=spts)
    out["bf_div_sector"] = ref.beamform(cddq, iq_d, 1, sx0, sx1, (0, 0, 0), spts, O.bf_config(f_number=1.5))
    out["bf_div_mv"] = ref.beamform(cddq, iq_d, 1, sx0, sx1, (0, 0, 0), spts,
                                    O.bf_config(f_number=1.5, combiner=2, mv_subarray=12))
    np.savez_compressed(HERE / "golden_bf.npz", **out)

    # ---- Doppler / strain ---------------------------------------------------------
    n_ens, n0, n1 = 10, 12, 30
    d_ax1 = np.linspace(0.020, 0.026, n1).astype(np.float32)
    ph = np.exp(-1j * 0.35 * np.arange(n_ens))[:, None, None] * np.exp(-1j * 0.85 * np.arange(n1))[None, None, :]
    clutter = 8.0 * np.exp(1j * 0.02 * np.arange(n_ens))[:, None, None]
    noise = rng.normal(size=(n_ens, n0, n1)) + 1j * rng.normal(size=(n_ens, n0, n1))
    ens = (clutter + 2.0 * ph + 0.2 * noise).astype(np.complex64)
    dop = {"ens": ens, "ax1": d_ax1}
    for wt, order in [(0, 1), (1, 1), (1, 2), (2, 0)]:
        dc = O.doppler_config(wall_filter=wt, polynomial_order=order)
        v, p, var, valid, nyq = ref.color_flow(ens, d_ax1, 5e6, 5000.0, 1540.0, dc)
        key = f"w{wt}o{order}"
        dop.update({f"cf_vel_{key}": v, f"cf_pow_{key}": p, f"cf_var_{key}": var, f"cf_valid_{key}": valid,
                    f"cf_nyq_{key}": np.float32(nyq), f"wall_{key}": ref.wall_filter(ens, d_ax1, wt, order),
                    f"pd_{key}": ref.power_doppler(ens, d_ax1, wt, order)})
    dc = O.doppler_config(loupas=0, kernel_axial=2, kernel_lateral=0, coherence_threshold=0.1)
    v, p, var, valid, _ = ref.color_flow(ens, d_ax1, 5e6, 5000.0, 1540.0, dc)
    dop.update(cf_vel_kasai=v, cf_valid_kasai=valid)
    a = (rng.normal(size=(n0, 40)) + 1j * rng.normal(size=(n0, 40))).astype(np.complex64)
    b = (np.roll(a, 3, axis=1) * np.exp(-0.4j)).astype(np.complex64)
    s_ax1 = np.linspace(0.02, 0.03, 40).astype(np.float32)
    ax_d, corr = ref.displacement(a, b, s_ax1, 5e6, 1540.0, 4, 1, 5)
    dop.update(disp_a=a, disp_b=b, disp_ax1=s_ax1, disp_axial=ax_d, disp_corr=corr,
               strain=ref.strain(ax_d, s_ax1, 9))
    np.savez_compressed(HERE / "golden_doppler.npz", **dop)

    # ---- post-processing ------------------------------------------------------------
    frame = out["bf_das"]
    post = {"frame": frame, "rf_frame": out["bf_rf"]}
    post["env_iq"] = ref.envelope(frame, 0, ax0, ax1, (0, 0, 0), pts, 5e6)
    post["env_rf"] = ref.envelope(out["bf_rf"], 0, ax0, ax1, (0, 0, 0), pts, 0.0)
    post["tgc"] = ref.apply_tgc(post["env_iq"], 0, ax0, ax1, (0, 0, 0), pts, 0.5, 5e6)
    post["log"] = ref.log_compress(post["tgc"], 50.0, 2.0, -1.0)
    post["log_ref"] = ref.log_compress(post["tgc"], 40.0, 0.0, float(post["tgc"].max() * 0.5))
    img = np.abs(rng.normal(size=(20, 36))).astype(np.float32)
    post["sc_img"] = img
    post["sc_sector"], post["sc_sector_ext"] = ref.scan_convert(img, 1, sx0, sx1, (0, 0, 0), spts, 50, 40, -1.0)
    post["sc_cart"], post["sc_cart_ext"] = ref.scan_convert(post["env_iq"], 0, ax0, ax1, (0, 0, 0), pts, 33, 47, 0.0)
    np.savez_compressed(HERE / "golden_post.npz", **post)

    # ---- image metrics, computed by the reference's own metrics module ---------------
    import importlib.util
    import types
    spec = importlib.util.spec_from_file_location("ref_metrics", REF_DIR / "python" / "usx" / "metrics.py")
    rm = importlib.util.module_from_spec(spec)
    sys.modules["ref_metrics"] = rm
    spec.loader.exec_module(rm)
    grid = types.SimpleNamespace(axis0=ax0, axis1=ax1)
    s = rm.summarize(post["env_iq"], grid, lesion_xz=(0.0, 0.014), lesion_radius=0.002, wire_xz=(-0.003, 0.010),
                     speckle_xz=(0.003, 0.018), speckle_half=(0.002, 0.002))
    keys = sorted(s)
    np.savez_compressed(HERE / "golden_metrics.npz", env=post["env_iq"],
                        grid=np.array([-0.006, 0.006, 16, 0.006, 0.022, 40], np.float64),
                        keys=np.array(keys), values=np.array([s[k] for k in keys], np.float64))

    for f in sorted(HERE.glob("golden_*.npz")):
        print(f"{f.name}: {f.stat().st_size / 1024:.0f} KB")


if __name__ == "__main__":
    main()
