"""Benchmark of the usx imaging path on one GB300.

Workload (the headline configuration): 128-element 5 MHz linear probe, 75
plane waves at -16..16 deg, 100,000-scatterer seeded speckle phantom with three
2-4 mm cysts, 60 mm depth (2073 samples at 20 MHz), IQ (75, 128, 2073)
complex64 beamformed onto a 512 x 1024 grid with minimum variance (subarray
64, diagonal loading tr(R)/(100 L), range averaging +/-2, f-number 1.5).

A step is one frame. `value` is frames/s with the IQ resident in HBM (159 MB,
larger than the 129 MB L2, so no flush is needed between steps); `e2e` is the
same metric through the public API (`usx.ImagingPipeline.process_frame` on a
host RF ChannelData: host-to-device copy of the RF, demodulation, beamforming,
device-to-host copy of the frame). The phantom is simulated on the GPU by the
project's own simulator at start-up (synthetic data; no dataset is used).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the reference's own CPU implementation of the same
beamformer (the reference library built from its sources where present, else
the CPU oracle port) on all host cores over a bounded sample of lines.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "ultrasound-engine_gb300"
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(PKG / "python"))

METRIC = "frames/s, 128ch 75-PW 512×1024: learned vs plain MV on 1 GB300 at ΔgCNR≤0.01"
N_EL, N_TX, N_SMP = 128, 75, 2073
N0, N1 = 512, 1024
FS, F0, C0 = 20e6, 5e6, 1540.0
MV_KW = dict(f_number=1.5, combiner=2, mv_subarray=64, mv_diagonal_loading=0.01, mv_range_average=2)
LEARNED_KW = dict(MV_KW, combiner=3)
WORKLOADS = {
    "learned": LEARNED_KW,   # learned MV with plain-MV fallback (the headline), plain MV timed beside it
    "mv": MV_KW,             # the fast plain MV (--mv-mode: FP32 lag recurrence by default, or tensor cores)
    "mv_exact": MV_KW,       # FP32 in the reference's operation order
    "das": dict(f_number=1.5),
    "cf": dict(f_number=1.5, coherence_factor=1),
    "dmas": dict(f_number=1.5, combiner=1),
}
CYSTS = ((-0.010, 0.025, 0.002), (0.0, 0.035, 0.003), (0.010, 0.045, 0.004))


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def workload_setup(n_scat: int = 100_000):
    """Probe, acquisition, transmits, grid and phantom of the headline workload (host objects)."""
    import usx
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = N_EL, 300e-6, 270e-6
    probe.center_frequency, probe.bandwidth = F0, 0.6
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.06, medium=medium, samples_per_wavelength=FS / F0)
    assert acq.n_samples == N_SMP
    cfg = usx.SimulatorConfig()
    sim = usx.Simulator(probe, medium, acq, cfg)
    txs = sim.make_plane_waves(usx.angles_deg(-16, 16, N_TX))
    half = 0.5 * probe.aperture_width()
    ph = usx.Phantom.speckle_box(-half * 1.1, half * 1.1, 0.004, 0.062, 0.0, n_scat, 2026)
    for x, z, r in CYSTS:
        ph.scale_amplitude_in_circle(usx.Vec3(x, 0.0, z), r, 0.0)
    grid = usx.grid_for(probe, 0.005, 0.060, N0, N1)
    return usx, probe, medium, acq, sim, txs, ph, grid


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled in the background
    during the timed region: through NVML (read-only queries, every 20 ms)
    where libnvidia-ml loads, else by running nvidia-smi every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits, in the order of the names in summary().
    BITS = (0x8, 0x40, 0x20, 0x4)

    def __init__(self, device: int = 0):
        self.device = device
        self.rows = []
        self.source = None
        self._stop = threading.Event()
        self._t = None
        self._nvml = self._open_nvml()

    def _open_nvml(self):
        import ctypes
        try:
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = ctypes.c_void_p()
            # The CUDA device's own PCI address (NVML's indices need not follow
            # CUDA_VISIBLE_DEVICES), else NVML's index.
            bus = None
            try:
                import torch
                p = torch.cuda.get_device_properties(self.device)
                bus = "%04x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)
            except Exception:
                bus = None
            if bus is None or lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(h)) != 0:
                if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(self.device), ctypes.byref(h)) != 0:
                    return None
            fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
            return lib, h, fn
        except (OSError, AttributeError):
            return None

    def _sample_nvml(self):
        import ctypes
        lib, h, reasons_fn = self._nvml
        sm, mx, mw, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm)) != 0:        # NVML_CLOCK_SM
            return None
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        lib.nvmlDeviceGetPowerUsage(h, ctypes.byref(mw))
        reasons_fn(h, ctypes.byref(rs))
        flags = ["Active" if rs.value & b else "Not Active" for b in self.BITS]
        return [str(sm.value), str(mx.value), f"{mw.value / 1000:.1f}"] + flags

    def _run(self):
        while not self._stop.is_set():
            row = None
            if self._nvml is not None:
                try:
                    row = self._sample_nvml()
                    self.source = "nvml"
                except Exception:
                    row = None
            if row is None:
                try:
                    out = subprocess.run(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                    if out.returncode == 0 and out.stdout.strip():
                        row = [v.strip() for v in out.stdout.strip().split(",")]
                        self.source = "nvidia-smi"
                except Exception:
                    pass
            if row is not None:
                self.rows.append(row)
            self._stop.wait(0.02 if self.source == "nvml" else 0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows), "source": self.source}


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12  # 152 SMs x 128 FP32 lanes x FMA x 2.07 GHz


def das_active_ops(grid_pts: np.ndarray, txs, probe, f_number: float) -> float:
    """Active (pixel, channel, transmit) triples of the delay-and-sum: receive
    aperture |x_e - x_p| < z / (2 F#) times transmits whose illuminated band
    (firing aperture shifted by z tan(angle), widened by the diffraction
    width, Tukey 0.4) covers the pixel (reference beamformer.cpp:238-288)."""
    x, z = grid_pts[:, 0].astype(np.float64), grid_pts[:, 2].astype(np.float64)
    ex = (np.arange(N_EL) - 0.5 * (N_EL - 1)) * probe.pitch
    half = 0.5 * z / f_number
    lo = np.maximum(0, np.ceil(0.5 * (N_EL - 1) + (x - half) / probe.pitch))
    hi = np.minimum(N_EL - 1, np.floor(0.5 * (N_EL - 1) + (x + half) / probe.pitch))
    n_act = np.maximum(0, hi - lo + 1)
    lam = C0 / F0
    n_tx = np.zeros_like(x)
    for t in txs:
        ap = np.asarray(t.apodization)
        on = np.nonzero(ap > 0)[0]
        if on.size == 0:
            continue
        x_lo, x_hi = ex[on[0]], ex[on[-1]]
        shift = z * np.tan(t.angle)
        aperture = max(x_hi - x_lo, probe.pitch)
        diff = np.clip(z / aperture, 0.5, 20.0) * lam
        a, b = x_lo + shift - diff, x_hi + shift + diff
        n_tx += np.abs(x - 0.5 * (a + b)) < 0.5 * (b - a)
    return float(np.sum(n_act * n_tx))


def mv_flops_per_frame(grid_pts: np.ndarray, cfg: dict) -> float:
    """Algorithmic FLOPs of minimum variance over the grid: covariance
    4 L^2 n_snap + Cholesky (4/3) L^3 + solves and apply 16 L^2 per pixel, with
    L and n_snap from the reference's clamp rule and the pixel's aperture."""
    z = grid_pts[:, 2]
    x = grid_pts[:, 0]
    ex = (np.arange(N_EL) - 0.5 * (N_EL - 1)) * 300e-6
    half = 0.5 * z / cfg["f_number"]
    n_act = (np.abs(ex[None, :] - x[:, None]) < half[:, None]).sum(1)
    L = np.clip(np.minimum(cfg["mv_subarray"], np.maximum(2, n_act // 2)), 2, None).astype(np.float64)
    n_snap = (2 * cfg["mv_range_average"] + 1) * (n_act - L + 1)
    ok = n_act >= 4
    f = 4 * L ** 2 * n_snap + (4.0 / 3.0) * L ** 3 + 16 * L ** 2
    return float(np.sum(f[ok]))


def plane_wave_table(angles: np.ndarray, n_el: int = N_EL, pitch: float = 300e-6, width: float = 270e-6,
                     c: float = C0):
    """Plane-wave delays and Hann transmit apodisation over the whole aperture,
    the reference's compute_transmit_delays (core/src/geometry.cpp:17-80) for
    PlaneWave with origin 0, restated in float32 for the CPU arm."""
    import ctypes
    libm = ctypes.CDLL("libm.so.6")  # the C library's sinf/cosf, as the reference's std::sin/std::cos
    for fn in (libm.sinf, libm.cosf):
        fn.argtypes, fn.restype = [ctypes.c_float], ctypes.c_float
    f = np.float32
    ex = ((np.arange(n_el, dtype=f) - f(0.5) * f(n_el - 1)) * f(pitch)).astype(f)
    half = f(0.5) * (f(n_el - 1) * f(pitch) + f(width))
    two_pi = f(2.0) * f(np.pi)
    apod = np.zeros(n_el, f)
    for i, x in enumerate(ex):
        u = x / max(half, f(1e-9))
        if -1 <= u <= 1:  # window_value(Hann, u), core/src/types.cpp:126-148
            t = f(0.5) * (u + f(1))
            apod[i] = f(0.5) * (f(1) - f(libm.cosf(two_pi * t)))
    sin = np.array([libm.sinf(float(a)) for a in angles], f)
    delays = np.where(apod[None, :] > 0, ex[None, :] * sin[:, None] / f(c), f(0)).astype(f)
    return delays, np.repeat(apod[None, :], len(angles), 0)


def baseline_lines(threads: int) -> np.ndarray:
    """Lateral lines of the CPU sample: two per host thread (the reference's
    beamformer splits its work across threads by blocks of pixels), evenly
    spread over the grid, at least 32."""
    n = int(min(N0, max(32, 2 * threads)))
    return np.linspace(0, N0 - 1, n).round().astype(int)


def cpu_baseline_mv(iq: np.ndarray, pts: np.ndarray, angles: np.ndarray, delays: np.ndarray, apod: np.ndarray,
                    fs: float, n_samples: int, prf: float, lines: np.ndarray, threads: int):
    """Time the CPU minimum variance on the given lateral lines; returns (s, kind)."""
    from oracle import oracle as O
    pr = O.probe(N_EL, 300e-6, 270e-6, 5e-3, F0, 0.6)
    oacq = O.acquisition(fs=fs, n_samples=n_samples, t0=0.0, prf=prf)
    n_tx = len(angles)
    tx = O.TxSet(np.ones(n_tx, np.int32), np.asarray(angles, np.float32),
                 np.tile([0, 0, 0.03], (n_tx, 1)).astype(np.float32), np.zeros((n_tx, 3), np.float32),
                 np.asarray(delays, np.float32), np.asarray(apod, np.float32))
    cd = O.channel_desc(pr, O.medium(), oacq, tx, is_iq=True, fdem=F0)
    sub = np.ascontiguousarray(pts.reshape(N0, N1, 3)[lines].reshape(-1, 3), dtype=np.float32)
    if O.REF_SO.exists():
        ref = O.RefLib()
        kind = "reference"
        axis1 = sub.reshape(len(lines), N1, 3)[0, :, 2]
        t = time.perf_counter()
        ref.beamform(cd, iq, 0, sub[::N1, 0], axis1, (0, 0, 0), sub, O.bf_config(**MV_KW))
        dt = time.perf_counter() - t
    else:
        orc = O.Lib("oracle")
        orc.set_threads(threads)
        kind = "port"
        t = time.perf_counter()
        orc.beamform(cd, iq, sub, len(lines), N1, O.bf_config(**MV_KW))
        dt = time.perf_counter() - t
    return dt, kind


def reference_workload():
    """The headline acquisition's geometry for the CPU arm, built with numpy
    alone (this engine's library is not loaded by the reference arm): 75
    plane waves at -16..16 deg, 2073 samples at 20 MHz, the 512 x 1024 grid
    over the aperture and z = 5-60 mm."""
    f = np.float32
    angles = np.deg2rad(np.linspace(-16, 16, N_TX)).astype(f)
    delays, apod = plane_wave_table(angles)
    half = f(0.5) * (f(N_EL - 1) * f(300e-6) + f(270e-6))
    ax0 = np.array([-half + (half - -half) * f(i) / f(N0 - 1) for i in range(N0)], f)
    ax1 = np.array([f(0.005) + (f(0.060) - f(0.005)) * f(i) / f(N1 - 1) for i in range(N1)], f)
    pts = np.zeros((N0, N1, 3), f)
    pts[:, :, 0] = ax0[:, None]
    pts[:, :, 2] = ax1[None, :]
    return angles, delays, apod, pts.reshape(-1, 3)


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    threads = int(os.environ["OMP_NUM_THREADS"])
    angles, delays, apod, pts = reference_workload()
    rng = np.random.default_rng(1)
    # The CPU minimum variance does the same work whatever the sample values
    # (every pixel forms its covariance and runs its Cholesky), so the arm
    # beamforms seeded random IQ of the workload's shape: the GPU arm's
    # simulated acquisition does not exist yet when this arm runs.
    iq = (rng.standard_normal((N_TX, N_EL, N_SMP), dtype=np.float32)
          + 1j * rng.standard_normal((N_TX, N_EL, N_SMP), dtype=np.float32)).astype(np.complex64)
    lines = baseline_lines(threads) if args.lines >= N0 else np.linspace(0, N0 - 1, args.lines).round().astype(int)
    times = []
    for i in range(args.warmup + args.steps):
        dt, kind = cpu_baseline_mv(iq, pts, angles, delays, apod, FS, N_SMP, 5000.0, lines, threads)
        if i >= args.warmup:
            times.append(dt)
    step_s = float(np.mean(times))
    v = len(lines) / N0 / step_s
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "frames/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded random IQ of the workload's shape)",
            "config": {"workload": f"{args.workload}_75pw_512x1024",
                       "beamformer": dict(WORKLOADS.get(args.workload, {})), "n_tx": N_TX, "n_ch": N_EL, "grid": [N0, N1],
                       "step": f"{len(lines)} of {N0} lateral lines (1/{N0 // len(lines)} frame); "
                               "value = frames/s = lines per second / 512",
                       "reference_path": "the reference has no learned combiner: its minimum variance "
                                         "(combine_mv_windowed, beamformer.cpp:137-214) on the same geometry"},
            "cpu_baseline": {"value": v, "unit": "frames/s", "cores": threads, "kind": kind,
                             "sample": f"{len(lines)} of {N0} lateral lines per step, full depth "
                                       f"({len(lines) * N1} pixels), {threads} threads",
                             "s_per_line": step_s / len(lines)},
            "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


WEIGHTS = PKG / "weights" / "learned_mv_128ch_l64.bin"
# DRAM bytes per launch of the dominant kernels from one ncu capture of the
# same workload (profiles/ holds the summaries these come from), scaled to a
# full 512-line frame where the capture was a subset of lines.
TRAFFIC_PER_FRAME = {
    # profiles/lmv_subspace_gram_kernel_7beams_64x1024.md: 95.39 MB read + 9.67 MB written for
    # the first 64 of 512 lines, scaled by 8 (deeper lines read wider apertures: a lower bound).
    "lmv_subspace_gram_kernel": 8 * (95.388e6 + 9.666e6),
}


def timed(stream, fn, steps: int):
    """Device time (ms) of `steps` calls of fn on `stream`, CUDA events around."""
    import torch
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        fn()
    ev1.record(stream)
    ev1.synchronize()
    return ev0.elapsed_time(ev1)


def subspace_flops_per_frame(grid_pts: np.ndarray, nb: int) -> float:
    """Algorithmic FLOPs of the learned-subspace refinement over the grid."""
    z, x = grid_pts[:, 2], grid_pts[:, 0]
    ex = (np.arange(N_EL) - 0.5 * (N_EL - 1)) * 300e-6
    n_act = (np.abs(ex[None, :] - x[:, None]) < 0.5 * z[:, None] / MV_KW["f_number"]).sum(1).astype(np.float64)
    L = np.clip(np.minimum(MV_KW["mv_subarray"], np.maximum(2, n_act // 2)), 2, None)
    n_d = 2 * MV_KW["mv_range_average"] + 1
    K = n_d * (n_act - L + 1)
    k = np.minimum(nb, L) + 1
    f = 8 * K * (L + k * (k + 1) / 2) + 8 * n_d * n_act * np.minimum(nb, L)
    return float(np.sum(f[n_act >= 4]))


def kernel_roofline(prof: dict, frames: int, pts: np.ndarray, txs, probe, peaks: dict,
                    refine_beams: int = -1, mv_mode: int = 1) -> dict:
    """Roofline of the dominant kernel of the timed region: algorithmic work
    per frame over that kernel's device time per frame (CUDA events on the
    launching stream)."""
    if not prof:
        return {"kernel": None, "bound": None, "achieved": None, "peak": None, "unit": None, "frac": None,
                "traffic": None}
    per_frame = {k: v[0] / frames for k, v in prof.items()}
    kname = max(per_frame, key=per_frame.get)
    kms = per_frame[kname]
    out = {"kernel": kname, "kernel_ms_per_frame": kms,
           "kernels_ms_per_frame": per_frame,
           "launches_per_frame": {k: v[1] / frames for k, v in prof.items()}}
    base = kname.split("(")[0]
    if base.startswith("mv") and mv_mode == 3:
        flops = mv_flops_per_frame(pts, MV_KW)
        achieved = flops / (kms / 1e3) / 1e12
        out.update(bound="fp32", achieved=achieved, peak=FP32_NOMINAL_TFLOPS, unit="TFLOP/s",
                   algorithmic_gflop_per_frame=flops / 1e9,
                   note="the reference formulation's flops (covariance 4 L^2 n_snap + Cholesky 4/3 L^3 + "
                        "solves 16 L^2 per pixel; the lag recurrence forms the covariance with fewer); "
                        "peak = nominal FP32")
    elif base.startswith("mv"):
        flops = mv_flops_per_frame(pts, MV_KW)
        achieved = flops / (kms / 1e3) / 1e12
        out.update(bound="tensor", achieved=achieved, peak=peaks["bf16_tflops_sustained"], unit="TFLOP/s",
                   algorithmic_gflop_per_frame=flops / 1e9,
                   note="covariance 4 L^2 n_snap + Cholesky 4/3 L^3 + solves 16 L^2 per pixel; "
                        "peak = cuBLAS bf16 sustained (measured)")
    elif base.startswith("das"):
        ops = das_active_ops(pts, txs, probe, 1.5)
        flops = 20.0 * ops
        achieved = flops / (kms / 1e3) / 1e12
        hbm = (8.0 * N_TX * N_EL * N_SMP + 8.0 * len(pts)) / (kms / 1e3) / 1e9
        out.update(bound="fp32", achieved=achieved, peak=FP32_NOMINAL_TFLOPS, unit="TFLOP/s",
                   algorithmic_gflop_per_frame=flops / 1e9, compulsory_hbm_gbs=hbm,
                   hbm_frac=hbm / peaks["hbm_gbs"],
                   note="20 FP32 flops per active (pixel, channel, transmit); peak = nominal FP32 "
                        "(152 SMs x 128 lanes x FMA x 2.07 GHz); compulsory HBM bytes = IQ + frame")
    elif base.startswith("lmv_subspace"):  # the Gram stage dominates; the per-pixel solve is ~0.2 ms
        nb = min(7, 1 + max(0, refine_beams))
        flops = subspace_flops_per_frame(pts, nb)
        achieved = flops / (kms / 1e3) / 1e12
        out.update(bound="fp32", achieved=achieved, peak=FP32_NOMINAL_TFLOPS, unit="TFLOP/s",
                   algorithmic_gflop_per_frame=flops / 1e9,
                   note="per pixel: 8 (L + k(k+1)/2) flops per snapshot (network-direction projection, "
                        "k = beams + 1 Gram entries) + 8 flops per beam and range-row sample (prefix "
                        "sums); peak = nominal FP32")
    elif base.startswith("mlp"):
        flops = 2.0 * len(pts) * sum(a * b for a, b in zip((256, 256, 256, 256), (256, 256, 256, 128)))
        achieved = flops / (kms / 1e3) / 1e12
        out.update(bound="tensor", achieved=achieved, peak=peaks["bf16_tflops"], unit="TFLOP/s",
                   algorithmic_gflop_per_frame=flops / 1e9)
    else:
        out.update(bound=None, achieved=None, peak=None, unit=None)
    out["frac"] = (out["achieved"] / out["peak"]) if out.get("achieved") and out.get("peak") else None
    tr = TRAFFIC_PER_FRAME.get(base)
    out["traffic"] = (tr / max(1.0, out["launches_per_frame"][kname])) if tr else None
    out["peak_source"] = peaks["source"]
    return out


def run_ours(args) -> None:
    import torch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    os.environ["USX_DEVICE"] = str(local)
    from usx import capi

    usx, probe, medium, acq, sim, txs, ph, grid = workload_setup()
    # Synthetic acquisition through the public API (GPU simulator + host copy).
    raw = sim.simulate(txs, ph)
    rf_host = np.asarray(raw.rf)
    ctx = capi.Context(local)
    tx = [dict(type=1, angle=t.angle, delays=t.delays, apodization=t.apodization) for t in txs]
    ch_rf = capi.Channel(capi.Probe(N_EL, probe.pitch, probe.element_width, probe.elevation_height, F0,
                                    probe.bandwidth),
                         capi.Medium(medium.speed_of_sound, medium.attenuation, medium.density),
                         capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf), tx)
    ch_iq = capi.Channel(ch_rf.desc.probe, ch_rf.desc.medium, ch_rf.desc.acq, tx, is_iq=True, fdem=F0)
    d_rf = torch.from_numpy(rf_host).cuda()
    d_iq = torch.empty((N_TX, N_EL, N_SMP), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()  # the context works on its own stream
    ctx.demodulate(ch_rf, capi.demod_config(), d_rf.data_ptr(), d_iq.data_ptr())
    ctx.synchronize()
    n0 = args.lines
    pts = np.asarray(grid.points).reshape(N0, N1, 3)[:n0].reshape(-1, 3)
    cgrid = capi.Grid(0, np.asarray(grid.axis0)[:n0], np.asarray(grid.axis1), pts)
    bkw = WORKLOADS[args.workload]
    frame = torch.empty((n0, N1), dtype=torch.complex64, device="cuda")
    stream = torch.cuda.ExternalStream(ctx.stream())

    extra = {}
    mlp = None
    if args.workload == "learned":
        from usx import learned
        if not WEIGHTS.exists():
            raise SystemExit(f"bench: the learned workload needs the trained network {WEIGHTS}")
        mlp = learned.load_mlp(ctx, WEIGHTS)
        gate = learned.trained_gate(WEIGHTS) if args.gate is None else args.gate
        refine = learned.trained_refine(WEIGHTS) if args.refine is None else args.refine
        share = learned.trained_share_gate(WEIGHTS) if args.share_gate is None else args.share_gate
        level = learned.trained_level_gate(WEIGHTS) if args.level_gate is None else args.level_gate
        window = learned.trained_level_window(WEIGHTS)
        # Plain minimum variance (tensor-core solver) on the same frame, timed first.
        plain = ctx.plan(ch_iq, cgrid, capi.bf_config(**MV_KW))
        plain.set_mv_mode(args.mv_mode)
        plain.autotune(d_iq.data_ptr(), frame.data_ptr(), repeats=1)
        for _ in range(args.warmup):
            plain.execute(d_iq.data_ptr(), frame.data_ptr())
        ctx.synchronize()
        plain_ms = timed(stream, lambda: plain.execute(d_iq.data_ptr(), frame.data_ptr()), args.steps)
        ref_frame = frame.clone()
        plain.close()
        # The tensor-core plain MV (tcgen05 BF16 covariance + refinement) on the
        # same frame, for reference beside the default solver.
        alt = None
        if args.mv_mode != 1:
            tc = ctx.plan(ch_iq, cgrid, capi.bf_config(**MV_KW))
            tc.set_mv_mode(1)
            tc.autotune(d_iq.data_ptr(), frame.data_ptr(), repeats=1)
            for _ in range(args.warmup):
                tc.execute(d_iq.data_ptr(), frame.data_ptr())
            ctx.synchronize()
            tc_ms = timed(stream, lambda: tc.execute(d_iq.data_ptr(), frame.data_ptr()), args.steps)
            tc.close()
            alt = {"value": world * args.steps / (tc_ms / 1e3) * N0 / n0, "unit": "frames/s",
                   "ms_per_step": tc_ms / args.steps * N0 / n0, "solver": "tensor"}
        plan = ctx.plan(ch_iq, cgrid, capi.bf_config(**bkw))
        plan.set_learned(mlp, gate)
        plan.set_learned_refine(refine)
        plan.set_learned_subspace(True, share)
        plan.set_learned_level_gate(level)
        plan.set_learned_level_window(*window)
        if args.mv_mode == 3:
            plan.set_mv_mode(3)   # the gated pixels take the same solver
        solver = {1: "tensor", 2: "tensor_mma", 3: "fp32_recurrence"}[args.mv_mode]
        extra["plain_mv"] = {"value": world * args.steps / (plain_ms / 1e3) * N0 / n0, "unit": "frames/s",
                             "ms_per_step": plain_ms / args.steps * N0 / n0, "solver": solver}
        if alt is not None:
            extra["plain_mv_tensor"] = alt
        extra["gate"] = gate
        extra["refine_beams"] = refine
        extra["share_gate"] = share
        extra["level_gate"] = level
        extra["level_window"] = list(window)
    else:
        plan = ctx.plan(ch_iq, cgrid, capi.bf_config(**bkw))
        if args.workload == "mv":
            plan.set_mv_mode(args.mv_mode)

    # The plan's autotuner picks the delay-and-sum launch shape on this acquisition.
    best, tune_ms = plan.autotune(d_iq.data_ptr(), frame.data_ptr(), repeats=2)
    extra["das_variant"] = {"chosen": capi.das_variants()[best], "ms_per_variant": tune_ms,
                            "variants": capi.das_variants()}
    for _ in range(args.warmup):
        plan.execute(d_iq.data_ptr(), frame.data_ptr())
    ctx.synchronize()
    if args.workload == "learned":
        plan.learned_stats()
    if world > 1:
        torch.distributed.barrier()
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(local) as clocks:
        ms = timed(stream, lambda: plan.execute(d_iq.data_ptr(), frame.data_ptr()), args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    ms_per_step = ms / args.steps
    value = world * args.steps / (ms / 1e3)
    if args.workload == "learned" and args.two_streams:
        # Two frames in flight: a second plan (same settings, same network) on
        # its own context and stream; frame i goes to plan i % 2.
        ctx2 = capi.Context(local)
        plan2 = ctx2.plan(ch_iq, cgrid, capi.bf_config(**bkw))
        plan2.set_learned(mlp, gate)
        plan2.set_learned_refine(refine)
        plan2.set_learned_subspace(True, share)
        plan2.set_learned_level_gate(level)
        plan2.set_learned_level_window(*window)
        if args.mv_mode == 3:
            plan2.set_mv_mode(3)
        plan2.set_variant(best)
        frame2 = torch.empty_like(frame)
        for _ in range(args.warmup):
            plan2.execute(d_iq.data_ptr(), frame2.data_ptr())
        ctx2.synchronize()
        s1, s2 = stream, torch.cuda.ExternalStream(ctx2.stream())
        ev0, ev_b, ev1 = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(), torch.cuda.Event(enable_timing=True))
        torch.cuda.synchronize()
        ev0.record(s1)
        s2.wait_event(ev0)
        for i in range(args.steps):
            (plan if i % 2 == 0 else plan2).execute(d_iq.data_ptr(), (frame if i % 2 == 0 else frame2).data_ptr())
        ev_b.record(s2)
        s1.wait_event(ev_b)
        ev1.record(s1)
        ev1.synchronize()
        ms2 = ev0.elapsed_time(ev1)
        extra["two_frames_in_flight"] = {"value": world * args.steps / (ms2 / 1e3) * N0 / n0, "unit": "frames/s",
                                         "ms_per_step": ms2 / args.steps * N0 / n0,
                                         "streams": 2, "note": "frames alternate between two plans on two streams"}
        plan2.close()
        ctx2.close()
    if args.workload == "learned":
        gated, pixels = plan.learned_stats()
        # The setting that meets the quality bar at the lowest fallback (from
        # the weights' held-out report), timed the same way on the same frame.
        rep = WEIGHTS.with_suffix(".json")
        bar = json.loads(rep.read_text()).get("at_bar") if rep.exists() else None
        if bar:
            plan.set_learned(mlp, float(bar["gate"]))
            plan.set_learned_subspace(True, float(bar["share_gate"]))
            plan.set_learned_level_gate(float(bar["level_gate"]))
            plan.set_learned_level_window(*bar.get("level_window", (0, 0)))
            for _ in range(args.warmup):
                plan.execute(d_iq.data_ptr(), frame.data_ptr())
            plan.learned_stats()
            bar_ms = timed(stream, lambda: plan.execute(d_iq.data_ptr(), frame.data_ptr()), args.steps)
            bg, bp = plan.learned_stats()
            extra["at_quality_bar"] = {"mode": bar["label"], "value": world * args.steps / (bar_ms / 1e3) * N0 / n0,
                                       "unit": "frames/s", "ms_per_step": bar_ms / args.steps * N0 / n0,
                                       "fallback_rate": bg / max(1, bp),
                                       "held_out_fallback_rate": bar.get("fallback_rate")}
            plan.set_learned(mlp, gate)
            plan.set_learned_subspace(True, share)
            plan.set_learned_level_gate(level)
            plan.set_learned_level_window(*window)
            plan.execute(d_iq.data_ptr(), frame.data_ptr())   # the headline frame again (quality fields below)
            plan.learned_stats()
        extra["fallback_rate"] = gated / max(1, pixels)
        extra["speedup_vs_plain_mv"] = (extra["plain_mv"]["ms_per_step"] / (ms_per_step * N0 / n0))
        if "plain_mv_tensor" in extra:
            extra["speedup_vs_plain_mv_tensor"] = (extra["plain_mv_tensor"]["ms_per_step"] / (ms_per_step * N0 / n0))
        extra["rel_l2_vs_plain_mv"] = float((frame - ref_frame).abs().pow(2).sum().sqrt()
                                            / ref_frame.abs().pow(2).sum().sqrt())
        rep = WEIGHTS.with_suffix(".json")
        if rep.exists():
            r = json.loads(rep.read_text())
            label = learned.Mode(gate=float(gate), share=float(share), level=float(level),
                                 window=tuple(window)).label
            ev = r.get("eval", {}).get(label)
            if ev:
                extra["held_out_quality"] = {
                    "mode": label, "phantoms": ev.get("phantoms"), "fallback_rate": ev.get("fallback_rate"),
                    "max_abs_delta_gcnr": ev.get("gcnr", {}).get("max_abs_delta"),
                    "max_rel_delta_lateral_fwhm": ev.get("lateral_fwhm_mm", {}).get("max_rel_delta"),
                    "max_rel_delta_axial_fwhm": ev.get("axial_fwhm_mm", {}).get("max_rel_delta"),
                    "meets_bar": r.get("meets_bar") if r.get("chosen") == label else None,
                    "source": str(rep.relative_to(ROOT))}
            ab = r.get("eval", {}).get("beams_only")
            if ab:
                extra["held_out_beams_only"] = {
                    "max_abs_delta_gcnr": ab.get("gcnr", {}).get("max_abs_delta"),
                    "max_rel_delta_lateral_fwhm": ab.get("lateral_fwhm_mm", {}).get("max_rel_delta"),
                    "rel_l2_mean": ab.get("rel_l2_mean")}

    peaks = load_peaks()
    launches_in_region = sum(n for _, n in prof.values())
    roofline = kernel_roofline(prof, args.steps, pts, txs, probe, peaks, extra.get("refine_beams", -1),
                               args.mv_mode)

    e2e = None if args.no_e2e else run_e2e(usx, grid, raw, rf_host, args, world,
                                           (gate, refine, share, level) if args.workload == "learned" else None)
    if bkw.get("combiner") == 2:
        fp64, failed = plan.mv_stats()
        roofline["mv_fp64_resolves_per_frame"] = fp64 / max(1, args.steps + args.warmup)
        roofline["mv_factorization_failures"] = failed

    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu:
            threads = os.cpu_count() or 1
            iq_host = d_iq.cpu().numpy()
            lines = baseline_lines(threads)
            dt, kind = cpu_baseline_mv(iq_host, np.asarray(grid.points), np.asarray([t.angle for t in txs]),
                                       np.asarray([t.delays for t in txs]), np.asarray([t.apodization for t in txs]),
                                       acq.sampling_frequency, acq.n_samples, acq.prf, lines, threads)
            cpu = {"value": len(lines) / N0 / dt, "unit": "frames/s", "cores": threads, "kind": kind,
                   "sample": f"minimum variance on {len(lines)} of {N0} lateral lines (full depth, "
                             f"{threads} threads) of the same acquisition, lines per second / 512",
                   "s_per_line": dt / len(lines)}
        frames_per_s = value * N0 / n0
        line = {"metric": METRIC, "value": frames_per_s, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step * N0 / n0, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (GPU-simulated 100k-scatterer cyst phantom)",
                "config": {"workload": f"{args.workload}_75pw_512x1024", "beamformer": bkw, "n_tx": N_TX,
                           "n_ch": N_EL, "grid": [N0, N1], "lines_timed": n0, "iq_bytes": int(d_iq.numel() * 8),
                           "l2": "inputs larger than L2 (159 MB IQ), no flush"},
                "gpu_launches": launches_in_region, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "clocks": clocks.summary()}
        line.update(extra)
        print(json.dumps(line))
    plan.close()
    if mlp is not None:
        mlp.close()
    ctx.close()


def run_stage(args) -> None:
    """Single-stage workloads on the headline acquisition: the forward
    simulator (`simulate`, args.scatterers scatterers x 128 elements x 75 plane
    waves, receive noise on) and the demodulator (`demod`, RF (75, 128, 2073)
    float32 -> IQ complex64, 33 taps, decimation 1)."""
    import torch
    from usx import capi
    torch.cuda.set_device(0)
    usx, probe, medium, acq, sim, txs, ph, grid = workload_setup(args.scatterers)
    ctx = capi.Context(0)
    tx = [dict(type=1, angle=t.angle, delays=t.delays, apodization=t.apodization) for t in txs]
    ch_rf = capi.Channel(capi.Probe(N_EL, probe.pitch, probe.element_width, probe.elevation_height, F0,
                                    probe.bandwidth),
                         capi.Medium(medium.speed_of_sound, medium.attenuation, medium.density),
                         capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf), tx)
    pos, amp = np.asarray(ph.positions), np.asarray(ph.amplitudes)
    sc = np.zeros((len(amp), 8), np.float32)
    sc[:, :3], sc[:, 3] = pos, amp
    d_sc = torch.from_numpy(sc).cuda()
    d_rf = torch.empty((N_TX, N_EL, N_SMP), dtype=torch.float32, device="cuda")
    d_iq = torch.empty((N_TX, N_EL, N_SMP), dtype=torch.complex64, device="cuda")
    z = torch.randn((N_TX, N_EL, N_SMP), device="cuda")
    torch.cuda.synchronize()
    scfg = capi.sim_config()
    stream = torch.cuda.ExternalStream(ctx.stream())
    stats = ctx.simulate(ch_rf, scfg, d_sc.data_ptr(), len(sc), z.data_ptr(), d_rf.data_ptr(), want_stats=True)
    if args.workload == "simulate":
        step = lambda: ctx.simulate(ch_rf, scfg, d_sc.data_ptr(), len(sc), z.data_ptr(), d_rf.data_ptr())
    else:
        step = lambda: ctx.demodulate(ch_rf, capi.demod_config(), d_rf.data_ptr(), d_iq.data_ptr())
    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(0) as clocks:
        ms = timed(stream, step, args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    peaks = load_peaks()
    per = {k: v[0] / args.steps for k, v in prof.items()}
    top = max(per, key=per.get)
    line = {"metric": f"{args.workload}: acquisitions/s", "value": args.steps / (ms / 1e3), "unit": "acquisitions/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "gpu_launches": sum(n for _, n in prof.values()), "clocks": clocks.summary()}
    if args.workload == "simulate":
        samples = stats[0]
        # Stage 1: a two-tap lerp-add (4 flops) per pulse tap per firing element
        # per (scatterer, transmit); stage 2: 4 flops per echo sample.
        import ctypes as C
        n_taps, half = C.c_int(), C.c_float()
        capi.lib().usx_cu_pulse(C.byref(ch_rf.desc.probe), C.byref(ch_rf.desc.acq), C.byref(scfg), None, 0,
                                C.byref(n_taps), C.byref(half))
        pulse_taps = n_taps.value
        n_fire = sum(int(np.count_nonzero(np.asarray(t.apodization))) for t in txs)
        flops = 4.0 * len(sc) * n_fire * pulse_taps + 4.0 * samples
        kms = per[top]
        line["config"] = {"workload": f"simulate_{len(sc)}scat_128el_75pw", "scatterers": len(sc),
                          "elements": N_EL, "transmits": N_TX, "samples": N_SMP}
        line["scatterer_element_samples_per_s"] = samples / (ms / args.steps / 1e3)
        line["roofline"] = {"kernel": top, "bound": "fp32", "achieved": flops / (kms / 1e3) / 1e12,
                            "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                            "frac": flops / (kms / 1e3) / 1e12 / FP32_NOMINAL_TFLOPS, "traffic": None,
                            "gflop_per_step": flops / 1e9, "echo_samples_per_step": samples,
                            "kernels_ms_per_step": per,
                            "note": "peak = nominal FP32 (152 SMs x 128 lanes x FMA x 2.07 GHz)"}
    else:
        nbytes = 4.0 * N_TX * N_EL * N_SMP + 8.0 * N_TX * N_EL * N_SMP
        kms = per[top]
        line["config"] = {"workload": "demod_75x128x2073_33taps_dec1",
                          "l2": "80 MB of RF in and 159 MB of IQ out per step (more than the 129 MB L2), no flush"}
        line["roofline"] = {"kernel": top, "bound": "hbm", "achieved": nbytes / (kms / 1e3) / 1e9,
                            "peak": peaks["hbm_gbs"], "unit": "GB/s",
                            "frac": nbytes / (kms / 1e3) / 1e9 / peaks["hbm_gbs"], "traffic": None,
                            "algorithmic_bytes": nbytes, "kernels_ms_per_step": per}
    print(json.dumps(line))
    ctx.close()


def _capi_channel(capi, probe, medium, acq, txs, is_iq=False, fdem=0.0):
    tx = [dict(type=int(t.type.value) if hasattr(t.type, "value") else 1, angle=t.angle,
               focus=(t.focus.x, t.focus.y, t.focus.z), origin=(t.origin.x, t.origin.y, t.origin.z),
               delays=t.delays, apodization=t.apodization) for t in txs]
    return capi.Channel(capi.Probe(probe.n_elements, probe.pitch, probe.element_width, probe.elevation_height,
                                   probe.center_frequency, probe.bandwidth),
                        capi.Medium(medium.speed_of_sound, medium.attenuation, medium.density),
                        capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf), tx, is_iq, fdem)


def _scatterers(ph) -> np.ndarray:
    pos, amp, vel = np.asarray(ph.positions), np.asarray(ph.amplitudes), np.asarray(ph.velocities)
    sc = np.zeros((len(amp), 8), np.float32)
    sc[:, :3], sc[:, 3], sc[:, 4:7] = pos, amp, vel
    return sc


def _stage_line(metric, unit, value, args, ms, prof, clocks, config, roofline, extra=None) -> dict:
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (GPU-simulated phantom)",
            "config": config, "gpu_launches": sum(n for _, n in prof.values()), "roofline": roofline,
            "kernels_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
            "clocks": clocks.summary()}
    line.update(extra or {})
    return line


def run_doppler(args) -> None:
    """Colour flow of uneven ensembles packed into one launch sequence: a
    3 mm vessel at 25 degrees (parabolic flow, 0.4 m/s peak, blood at 0.1 x the
    tissue amplitude, tissue moving at 5 mm/s), ensembles of 8, 12, 16 and 32
    pulses at 5 kHz, 3 plane waves per pulse, 32 ensembles; one step = the
    delay-and-sum of all 544 frames (one launch) + order-2 polynomial wall
    filter and Loupas velocity for all 32 ensembles (one launch sequence)."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = N_EL, 300e-6, 270e-6
    probe.center_frequency, probe.bandwidth = F0, 0.6
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.04, medium=medium, samples_per_wavelength=FS / F0)
    acq.prf = 5000.0
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    angles = usx.angles_deg(-5, 5, 3)
    lens = [8, 12, 16, 32] * 8
    n_max = max(lens)
    txs = sim.make_plane_waves(angles * n_max)
    ph = usx.phantoms.flow_phantom(probe, medium, vessel_depth=0.022, vessel_radius=0.003, angle_deg=25.0,
                                  peak_velocity=0.4, z_min=0.005, z_max=0.04)
    sc = _scatterers(ph)
    blood = np.linalg.norm(sc[:, 4:7], axis=1) > 0
    sc[blood, 3] *= 0.1 / max(1e-12, np.abs(sc[blood, 3]).mean() / max(1e-12, np.abs(sc[~blood, 3]).mean()))
    sc[~blood, 6] = 0.005                       # tissue drifting axially at 5 mm/s
    ctx = capi.Context(0)
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    n_ev, n_smp = len(txs), acq.n_samples
    d_sc = torch.from_numpy(sc).cuda()
    d_rf = torch.empty((n_ev, N_EL, n_smp), dtype=torch.float32, device="cuda")
    d_iq1 = torch.empty((n_ev, N_EL, n_smp), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.simulate(ch_rf, capi.sim_config(noise_db=-200.0), d_sc.data_ptr(), len(sc), None, d_rf.data_ptr())
    ctx.demodulate(ch_rf, capi.demod_config(), d_rf.data_ptr(), d_iq1.data_ptr())
    ctx.synchronize()
    # Pack the 32 ensembles (each the first n_e pulses) into one acquisition.
    n_frames_total = sum(lens)
    iq = torch.empty((3 * n_frames_total, N_EL, n_smp), dtype=torch.complex64, device="cuda")
    off, offsets = 0, []
    for n in lens:
        iq[3 * off:3 * (off + n)] = d_iq1[:3 * n]
        offsets.append(off)
        off += n
    del d_rf
    all_tx = [t for n in lens for t in txs[:3 * n]]
    ch_iq = _capi_channel(capi, probe, medium, acq, all_tx, is_iq=True, fdem=F0)
    n0, n1 = 256, 512
    grid = usx.grid_for(probe, 0.01, 0.035, n0, n1)
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), np.asarray(grid.points).reshape(-1, 3))
    plan = ctx.plan(ch_iq, cgrid, capi.bf_config(f_number=1.5))
    frames = torch.empty((n_frames_total, n0 * n1), dtype=torch.complex64, device="cuda")
    n_ens = len(lens)
    vel = torch.empty((n_ens, n0 * n1), device="cuda")
    pw, var = torch.empty_like(vel), torch.empty_like(vel)
    valid = torch.empty((n_ens, n0 * n1), dtype=torch.uint8, device="cuda")
    dcfg = capi.doppler_config(wall_filter=1, polynomial_order=2, loupas=1)
    axis1 = np.asarray(grid.axis1)

    def step():
        plan.execute_sequence(3, n_frames_total, iq.data_ptr(), frames.data_ptr(), n0 * n1)
        ctx.color_flow_batch(frames.data_ptr(), lens, offsets, n0, n1, axis1, F0, acq.prf / 3.0,
                             medium.speed_of_sound, dcfg, vel.data_ptr(), pw.data_ptr(), var.data_ptr(),
                             valid.data_ptr())

    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(0) as clocks:
        ms = timed(stream, step, args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    peaks = load_peaks()
    per = {k: v[0] / args.steps for k, v in prof.items()}
    flow = [k for k in per if k.startswith("flow") or k.startswith("wall") or k.startswith("power_gate")]
    flow_ms = sum(per[k] for k in flow)
    # Colour flow reads every packed frame once and writes four maps per ensemble.
    flow_bytes = 8.0 * n_frames_total * n0 * n1 + n_ens * n0 * n1 * (3 * 4 + 1)
    v = vel.cpu().numpy()
    inside = valid.cpu().numpy().astype(bool)
    das_ms = sum(v for k, v in per.items() if k.startswith("das"))
    das_flops = 20.0 * das_active_ops(np.asarray(grid.points).reshape(-1, 3), txs[:3], probe, 1.5) * n_frames_total
    roof = {"kernel": max(per, key=per.get), "bound": "fp32",
            "achieved": das_flops / (das_ms / 1e3) / 1e12 if das_ms else None, "peak": FP32_NOMINAL_TFLOPS,
            "unit": "TFLOP/s", "frac": das_flops / (das_ms / 1e3) / 1e12 / FP32_NOMINAL_TFLOPS if das_ms else None,
            "traffic": None, "note": "delay-and-sum of all packed frames (20 flops per active pixel-channel-"
                                     "transmit); peak = nominal FP32",
            "colour_flow": {"ms": flow_ms, "bytes": flow_bytes,
                            "achieved_gbs": flow_bytes / (flow_ms / 1e3) / 1e9 if flow_ms else None,
                            "hbm_frac": flow_bytes / (flow_ms / 1e3) / 1e9 / peaks["hbm_gbs"] if flow_ms else None}}
    line = _stage_line("colour-flow ensembles/s (32 uneven ensembles of 8-32 pulses x 3 PW, 256x512)",
                       "ensembles/s", n_ens * args.steps / (ms / 1e3), args, ms, prof, clocks,
                       {"workload": "doppler_32ens_8-32pulses_3pw_256x512", "frames_per_step": n_frames_total,
                        "events_per_step": 3 * n_frames_total},
                       roof, {"valid_fraction": float(inside.mean()),
                              "peak_velocity_valid_m_s": float(np.abs(v[inside]).max()) if inside.any() else None})
    print(json.dumps(line))
    plan.close()
    ctx.close()


def run_strain(args) -> None:
    """Elastography: a 4x-stiff 5 mm inclusion at 30 mm under 1% compression,
    one plane wave before and after; one step = two 256 x 1024 delay-and-sum
    frames, axial displacement tracking and least-squares strain (2 mm fit)."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = N_EL, 300e-6, 270e-6
    probe.center_frequency, probe.bandwidth = F0, 0.6
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.05, medium=medium, samples_per_wavelength=FS / F0)
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    txs = sim.make_plane_waves(usx.angles_deg(0, 0, 1))
    ctx = capi.Context(0)
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    ch_iq = _capi_channel(capi, probe, medium, acq, txs, is_iq=True, fdem=F0)
    n_smp = acq.n_samples
    iqs = []
    for strain in (0.0, 0.01):
        sc = _scatterers(usx.phantoms.elastography_phantom(probe, medium, strain=strain))
        d_sc = torch.from_numpy(sc).cuda()
        rf = torch.empty((1, N_EL, n_smp), device="cuda")
        iq = torch.empty((1, N_EL, n_smp), dtype=torch.complex64, device="cuda")
        torch.cuda.synchronize()
        ctx.simulate(ch_rf, capi.sim_config(noise_db=-200.0, enable_motion=0), d_sc.data_ptr(), len(sc), None,
                     rf.data_ptr())
        ctx.demodulate(ch_rf, capi.demod_config(), rf.data_ptr(), iq.data_ptr())
        ctx.synchronize()
        iqs.append(iq)
    n0, n1 = 256, 1024
    grid = usx.grid_for(probe, 0.012, 0.048, n0, n1)
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), np.asarray(grid.points).reshape(-1, 3))
    plan = ctx.plan(ch_iq, cgrid, capi.bf_config(f_number=1.5))
    fa = torch.empty((n0, n1), dtype=torch.complex64, device="cuda")
    fb = torch.empty_like(fa)
    axial = torch.empty((n0, n1), device="cuda")
    corr, strain_map = torch.empty_like(axial), torch.empty_like(axial)
    axis1 = np.asarray(grid.axis1)
    dz = float(axis1[1] - axis1[0])
    fit = max(3, int(round(0.002 / dz)) | 1)

    def step():
        plan.execute(iqs[0].data_ptr(), fa.data_ptr())
        plan.execute(iqs[1].data_ptr(), fb.data_ptr())
        ctx.axial_displacement(fa.data_ptr(), fb.data_ptr(), n0, n1, axis1, F0, medium.speed_of_sound, 8, 2, 8,
                               axial.data_ptr(), corr.data_ptr())
        ctx.axial_strain(axial.data_ptr(), n0, n1, axis1, fit, strain_map.data_ptr())

    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(0) as clocks:
        ms = timed(stream, step, args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    peaks = load_peaks()
    per = {k: v[0] / args.steps for k, v in prof.items()}
    track = sum(v for k, v in per.items() if k.startswith("displacement") or k.startswith("strain"))
    tbytes = 2 * 8.0 * n0 * n1 + 3 * 4.0 * n0 * n1
    s = strain_map.cpu().numpy()
    roof = {"kernel": "displacement_kernel + strain_kernel", "bound": "hbm",
            "achieved": tbytes / (track / 1e3) / 1e9 if track else None, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": (tbytes / (track / 1e3) / 1e9 / peaks["hbm_gbs"]) if track else None, "traffic": None,
            "note": "tracking kernels: two frames in, displacement, correlation and strain out"}
    mid = s[:, n1 // 4:3 * n1 // 4]
    line = _stage_line("strain maps/s (1% compression, 256x1024, 2 mm fit)", "maps/s", args.steps / (ms / 1e3),
                       args, ms, prof, clocks, {"workload": "strain_1pw_256x1024", "fit_samples": fit}, roof,
                       {"median_strain_background": float(np.median(mid))})
    print(json.dumps(line))
    plan.close()
    ctx.close()


BATCH_BEAMFORMERS = {
    "das": dict(f_number=1.5),
    "cf": dict(f_number=1.5, coherence_factor=1),
    "dmas": dict(f_number=1.5, combiner=1),
    "mv": MV_KW,
}


def cpu_leg_batch(iq0: np.ndarray, pts: np.ndarray, txs, probe, acq, gpu_lines: dict, line_idx, threads: int):
    """CPU side of the batched workload: the reference's CPU beamformers (its
    own build when present, else the oracle's port) timed on a sample of
    lateral lines and scaled to a frame, and the FP64 oracle on `line_idx` as
    the checker of each GPU beamformer's frame 0 (relative L2), beside the
    distance of the reference's own FP32 arithmetic (the oracle's f32
    restatement) from the FP64 oracle on the same lines."""
    from oracle import oracle as O
    pr = O.probe(N_EL, probe.pitch, probe.element_width, 5e-3, F0, probe.bandwidth)
    oacq = O.acquisition(fs=acq.sampling_frequency, n_samples=acq.n_samples, t0=acq.t0, prf=acq.prf)
    tx = O.TxSet(np.ones(len(txs), np.int32), np.asarray([t.angle for t in txs], np.float32),
                 np.tile([0, 0, 0.03], (len(txs), 1)).astype(np.float32), np.zeros((len(txs), 3), np.float32),
                 np.asarray([t.delays for t in txs], np.float32), np.asarray([t.apodization for t in txs], np.float32))
    cd = O.channel_desc(pr, O.medium(), oacq, tx, is_iq=True, fdem=F0)
    grid_pts = pts.reshape(N0, N1, 3)
    orc = O.Lib("oracle")
    orc.set_threads(threads)
    n_time = max(2, min(threads, 16))
    t_idx = np.linspace(0, N0 - 1, n_time).astype(int)
    sub_t = grid_pts[t_idx].reshape(-1, 3)
    sub_e = grid_pts[list(line_idx)].reshape(-1, 3)
    ref = O.RefLib() if O.REF_SO.exists() else None
    seconds, errors, ref_errors = {}, {}, {}
    for name, kw in BATCH_BEAMFORMERS.items():
        t = time.perf_counter()
        if ref is not None:
            ref.beamform(cd, iq0, 0, sub_t[::N1, 0], sub_t[:N1, 2], (0, 0, 0), sub_t, O.bf_config(**kw))
        else:
            orc.beamform(cd, iq0, sub_t, n_time, N1, O.bf_config(**kw))
        seconds[name] = (time.perf_counter() - t) * N0 / n_time
        want = orc.beamform(cd, iq0, sub_e, len(line_idx), N1, O.bf_config(**kw), prec="f64")
        ref32 = orc.beamform(cd, iq0, sub_e, len(line_idx), N1, O.bf_config(**kw), prec="f32")
        got = gpu_lines[name].astype(np.complex128)
        errors[name] = float(np.linalg.norm(got - want) / max(1e-300, np.linalg.norm(want)))
        ref_errors[name] = float(np.linalg.norm(ref32 - want) / max(1e-300, np.linalg.norm(want)))
    total = sum(seconds.values())
    cpu = {"value": len(seconds) / total, "unit": "frames/s", "cores": threads,
           "kind": "reference" if ref is not None else "port",
           "sample": f"{', '.join(seconds)} on {n_time} of {N0} lateral lines of frame 0, scaled to a frame",
           "seconds_per_frame": seconds}
    return cpu, errors, ref_errors


def run_batch(args) -> None:
    """Batched plain beamformers: 64 acquisitions of distinct seeded phantoms
    (100,000 scatterers each, three cysts of radius 2-4 mm, 75 plane waves at
    -16..16 degrees, 60 mm, simulated and demodulated on the GPU), beamformed
    onto 512 x 1024 by delay-and-sum, coherence-factor DAS, DMAS and minimum
    variance (L = 64, range averaging 2, loading tr(R) / (100 L); tensor-core
    covariance). Each beamformer's 64 frames are captured once into a CUDA
    graph (DAS, CF and DMAS as one batched launch sequence; MV as 64 frame
    executions, whose channel export is 0.5 GB a frame) and one step replays
    the four graphs. Reported per beamformer: frames/s and the relative L2
    error of frame 0 against the FP64 oracle on four lateral lines."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    n_frames = 64
    _, probe, medium, acq, _, txs, _, grid = workload_setup()
    stream = torch.cuda.Stream()
    ctx = capi.Context(0, stream=stream.cuda_stream)
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    ch_iq = _capi_channel(capi, probe, medium, acq, txs, is_iq=True, fdem=F0)
    half = 0.5 * probe.aperture_width()
    iq = torch.empty((n_frames, N_TX, N_EL, N_SMP), dtype=torch.complex64, device="cuda")
    d_rf = torch.empty((N_TX, N_EL, N_SMP), device="cuda")
    t_sim = time.perf_counter()
    for f in range(n_frames):
        ph = usx.Phantom.speckle_box(-half * 1.1, half * 1.1, 0.004, 0.062, 0.0, 100_000, 2026 + f)
        for x, z, r in CYSTS:
            ph.scale_amplitude_in_circle(usx.Vec3(x, 0.0, z), r, 0.0)
        d_sc = torch.from_numpy(_scatterers(ph)).cuda()
        with torch.cuda.stream(stream):
            ctx.simulate(ch_rf, capi.sim_config(noise_db=-200.0), d_sc.data_ptr(), len(d_sc), None,
                         d_rf.data_ptr())
            ctx.demodulate(ch_rf, capi.demod_config(), d_rf.data_ptr(), iq[f].data_ptr())
        ctx.synchronize()
    t_sim = time.perf_counter() - t_sim
    del d_rf
    pts = np.asarray(grid.points, np.float32).reshape(-1, 3)
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), pts)
    frames = torch.empty((n_frames, N0, N1), dtype=torch.complex64, device="cuda")
    iq_stride, fr_stride = N_TX * N_EL * N_SMP, N0 * N1
    line_idx = (0, 170, 341, 511)
    plans, graphs, lines0, prof_all = {}, {}, {}, {}
    for name, kw in BATCH_BEAMFORMERS.items():
        plan = ctx.plan(ch_iq, cgrid, capi.bf_config(**kw))
        if name == "mv":
            plan.set_mv_mode(args.mv_mode)
        with torch.cuda.stream(stream):
            plan.autotune(iq[0].data_ptr(), frames[0].data_ptr(), repeats=1)

        def run(plan=plan, name=name):
            if name == "mv":
                for f in range(n_frames):
                    plan.execute(iq[f].data_ptr(), frames[f].data_ptr())
            else:
                plan.execute_batch(n_frames, iq.data_ptr(), iq_stride, frames.data_ptr(), fr_stride)

        with torch.cuda.stream(stream):
            run()                                  # sizes the scratch arena
            stream.synchronize()
            capi.profile(ctx, True)
            capi.profile_reset(ctx)
            run()                                  # one direct pass: per-kernel device times
            stream.synchronize()
            prof_all[name] = capi.profile_read(ctx)
            capi.profile(ctx, False)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=stream):
                run()
            stream.synchronize()
            g.replay()
            stream.synchronize()
        lines0[name] = frames[0].cpu().numpy()[list(line_idx)]
        plans[name], graphs[name] = plan, g
    # Replays go to the current stream: every replay below runs on `stream`,
    # where the events are recorded.
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            for g in graphs.values():
                g.replay()
    stream.synchronize()
    per_bf = {}
    with ClockSampler(0) as clocks, torch.cuda.stream(stream):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(graphs) + 1)]
        torch.cuda.synchronize()
        ms = {n: 0.0 for n in graphs}
        for _ in range(args.steps):
            ev[0].record(stream)
            for i, g in enumerate(graphs.values()):
                g.replay()
                ev[i + 1].record(stream)
            ev[-1].synchronize()
            for i, n in enumerate(graphs):
                ms[n] += ev[i].elapsed_time(ev[i + 1])
    total_ms = sum(ms.values())
    for n in graphs:
        per_bf[n] = {"frames_per_s": n_frames * args.steps / (ms[n] / 1e3), "ms_per_frame": ms[n] / (n_frames * args.steps),
                     "graph_launches_per_step": 1}
    peaks = load_peaks()
    prof = {}
    for p in prof_all.values():
        for k, v in p.items():
            a = prof.setdefault(k, [0.0, 0])
            a[0] += v[0]
            a[1] += v[1]
    roof = kernel_roofline(prof, n_frames, pts, txs, probe, peaks)
    cpu = None
    if not args.no_cpu:
        cpu, errors, ref_errors = cpu_leg_batch(iq[0].cpu().numpy(), pts, txs, probe, acq, lines0, line_idx,
                                                os.cpu_count() or 1)
        for n, e in errors.items():
            per_bf[n]["fp64_oracle_rel_l2_frame0"] = e
            per_bf[n]["reference_fp32_rel_l2_vs_fp64_frame0"] = ref_errors[n]
    launches = sum(v[1] for v in prof.values()) * args.steps  # one pass of the four graphs per step
    line = {"metric": "beamformed frames/s, 64-frame batch of 128ch 75-PW 512x1024 (DAS, CF, DMAS, MV; one CUDA "
                      "graph per beamformer)",
            "value": len(graphs) * n_frames * args.steps / (total_ms / 1e3), "unit": "frames/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (64 GPU-simulated 100k-scatterer cyst phantoms, seeds 2026-2089)",
            "config": {"workload": "batch_64x_75pw_512x1024", "beamformers": BATCH_BEAMFORMERS,
                       "mv_solver": {1: "tensor", 2: "tensor_mma", 3: "fp32_recurrence"}[args.mv_mode],
                       "frames": n_frames, "iq_bytes": int(iq.numel() * 8),
                       "l2": "inputs larger than L2 (10.2 GB IQ), no flush"},
            "gpu_launches": launches, "graph_replays_per_step": len(graphs), "beamformers": per_bf,
            "roofline": roof, "cpu_baseline": cpu, "e2e": None, "clocks": clocks.summary(),
            "simulation_s": t_sim}
    print(json.dumps(line))
    for p in plans.values():
        p.close()
    ctx.close()


def run_post(args) -> None:
    """B-mode post-processing of a cine loop: 48 distinct 512 x 1024 IQ frames
    (192 MB, larger than L2), each through envelope (|IQ|), time-gain
    compensation (0.5 dB/cm/MHz at 5 MHz), 60 dB log compression against the
    frame's own maximum (found on the device; output in [0, 1]) and scan
    conversion to a 512 x 800 raster; one step = the whole loop through the C-ABI, one call per
    stage and frame as the reference's postprocess functions are called."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = N_EL, 300e-6, 270e-6
    n0, n1, n_frames, width, height = 512, 1024, 48, 512, 800
    grid = usx.grid_for(probe, 0.005, 0.045, n0, n1)
    pts = np.ascontiguousarray(np.asarray(grid.points, np.float32).reshape(-1, 3))
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), pts)
    ctx = capi.Context(0)
    g = torch.Generator(device="cuda").manual_seed(7)
    depth = torch.exp(-torch.linspace(0.0, 4.0, n1, device="cuda"))
    frames = torch.complex(torch.randn((n_frames, n0, n1), device="cuda", generator=g),
                           torch.randn((n_frames, n0, n1), device="cuda", generator=g)) * depth
    d_pts = torch.from_numpy(pts).cuda()
    env = torch.empty((n0, n1), device="cuda")
    tgc, logc = torch.empty_like(env), torch.empty_like(env)
    px = torch.empty((n_frames, height, width), device="cuda")
    torch.cuda.synchronize()

    def step():
        for f in range(n_frames):
            ctx.envelope(frames[f].data_ptr(), n0, n1, F0, env.data_ptr())
            ctx.apply_tgc(env.data_ptr(), n0, n1, d_pts.data_ptr(), 0.5, F0, tgc.data_ptr())
            ctx.log_compress(tgc.data_ptr(), n0 * n1, 60.0, 0.0, 0.0, logc.data_ptr())
            ctx.scan_convert(logc.data_ptr(), cgrid, width, height, 0.0, px[f].data_ptr())

    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        step()
    ctx.synchronize()
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(0) as clocks:
        ms = timed(stream, step, args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    peaks = load_peaks()
    per = {k: v[0] / args.steps for k, v in prof.items()}
    kern_ms = sum(per.values())
    n = n0 * n1
    # Per frame: envelope 8n in + 4n out; TGC 4n + 12n (points) in, 4n out; maximum 4n in;
    # log compression 4n in, 4n out; scan conversion 4n in (each sample at least once), 4 W H out.
    fbytes = 48.0 * n + 4.0 * width * height
    achieved = fbytes * n_frames / (kern_ms / 1e3) / 1e9 if kern_ms else None
    roof = {"kernel": max(per, key=per.get), "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
            "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"] if achieved else None, "traffic": None,
            "bytes_per_frame": fbytes,
            "note": "all post-processing kernels together: compulsory bytes per frame over their summed "
                    "device time; the TGC points and the previous stage's output are L2-resident"}
    px_h = px[-1].cpu().numpy()
    line = _stage_line("post-processed frames/s (512x1024 IQ -> 512x800 B-mode, 60 dB)", "frames/s",
                       n_frames * args.steps / (ms / 1e3), args, ms, prof, clocks,
                       {"workload": "post_48x512x1024_to_512x800", "frames_per_step": n_frames,
                        "l2": "inputs larger than L2 (192 MB IQ), no flush"},
                       roof, {"kernel_ms_per_frame": kern_ms / n_frames,
                              "mean_b_mode_level": float(px_h.mean())})
    line["data"] = "synthetic (complex Gaussian speckle with exponential depth decay)"
    print(json.dumps(line))
    ctx.close()


def run_sector(args) -> None:
    """Phased-array sector imaging: 64 elements, 2.5 MHz, pitch 0.2 mm, 31
    diverging waves over +/-45 degrees (virtual source 10 mm behind the
    array), a 100,000-scatterer phantom with two cysts to 80 mm; one step =
    delay-and-sum onto 256 beams x 1024 samples, envelope, 60 dB log
    compression and scan conversion to 800 x 800. The tensor-core minimum
    variance of the same frame is timed beside it."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    probe = usx.Probe()
    probe.n_elements, probe.pitch, probe.element_width = 64, 200e-6, 180e-6
    probe.center_frequency, probe.bandwidth = 2.5e6, 0.6
    medium = usx.Medium()
    acq = usx.presets.acquisition(probe, depth=0.082, medium=medium, samples_per_wavelength=4.0)
    sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
    txs = sim.make_diverging_waves(usx.angles_deg(-45, 45, 31), 0.01)
    ph = usx.Phantom.speckle_box(-0.06, 0.06, 0.004, 0.084, 0.0, 100_000, 2027)
    for x, z, r in ((-0.015, 0.04, 0.004), (0.02, 0.06, 0.005)):
        ph.scale_amplitude_in_circle(usx.Vec3(x, 0.0, z), r, 0.0)
    sc = _scatterers(ph)
    ctx = capi.Context(0)
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    ch_iq = _capi_channel(capi, probe, medium, acq, txs, is_iq=True, fdem=probe.center_frequency)
    n_ev, n_smp = len(txs), acq.n_samples
    d_sc = torch.from_numpy(sc).cuda()
    rf = torch.empty((n_ev, 64, n_smp), device="cuda")
    iq = torch.empty((n_ev, 64, n_smp), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.simulate(ch_rf, capi.sim_config(noise_db=-60.0), d_sc.data_ptr(), len(sc), None, rf.data_ptr())
    ctx.demodulate(ch_rf, capi.demod_config(), rf.data_ptr(), iq.data_ptr())
    ctx.synchronize()
    n0, n1 = 256, 1024
    grid = usx.ScanGrid.sector(float(np.deg2rad(-45.0)), float(np.deg2rad(45.0)), n0, 0.005, 0.08, n1,
                               usx.Vec3(0.0, 0.0, 0.0))
    pts = np.asarray(grid.points).reshape(-1, 3)
    cgrid = capi.Grid(1, np.asarray(grid.axis0), np.asarray(grid.axis1), pts)
    d_pts = torch.from_numpy(pts).cuda()
    frame = torch.empty((n0, n1), dtype=torch.complex64, device="cuda")
    env, logi = torch.empty((n0, n1), device="cuda"), torch.empty((n0, n1), device="cuda")
    W = H = 800
    img = torch.empty((H, W), device="cuda")
    fdem = probe.center_frequency

    def make(kw, mv=False):
        plan = ctx.plan(ch_iq, cgrid, capi.bf_config(**kw))
        if mv:
            plan.set_mv_mode(args.mv_mode)
        plan.autotune(iq.data_ptr(), frame.data_ptr(), repeats=1)
        return plan

    def step_with(plan):
        def step():
            plan.execute(iq.data_ptr(), frame.data_ptr())
            ctx.envelope(frame.data_ptr(), n0, n1, fdem, env.data_ptr())
            ctx.log_compress(env.data_ptr(), n0 * n1, 60.0, 0.0, -1.0, logi.data_ptr())
            ctx.scan_convert(logi.data_ptr(), cgrid, W, H, 0.0, img.data_ptr())
        return step

    stream = torch.cuda.ExternalStream(ctx.stream())
    das = make(dict(f_number=1.5))
    mvp = make(dict(f_number=1.5, combiner=2, mv_subarray=32, mv_diagonal_loading=0.01, mv_range_average=2),
               mv=True)
    results = {}
    for name, plan in (("mv", mvp), ("das", das)):
        step = step_with(plan)
        for _ in range(args.warmup):
            step()
        ctx.synchronize()
        capi.profile(ctx, True)
        capi.profile_reset(ctx)
        with ClockSampler(0) as clocks:
            ms = timed(stream, step, args.steps)
        results[name] = (ms, capi.profile_read(ctx), clocks)
        capi.profile(ctx, False)
    ms, prof, clocks = results["das"]
    per = {k: v[0] / args.steps for k, v in prof.items()}
    ops = 0.0  # active (pixel, channel, transmit) triples are not counted for diverging waves
    roof = {"kernel": max(per, key=per.get), "bound": None, "achieved": None, "peak": None, "unit": None,
            "frac": None, "traffic": None}
    mv_ms = results["mv"][0] / args.steps
    line = _stage_line("sector frames/s (64-el 2.5 MHz phased array, 31 diverging waves, 256x1024 -> 800x800)",
                       "frames/s", args.steps / (ms / 1e3), args, ms, prof, clocks,
                       {"workload": "sector_64el_31dw_256x1024_800x800", "beamformer": "das f#1.5"}, roof,
                       {"mv_tensor": {"value": 1e3 / mv_ms, "unit": "frames/s", "ms_per_step": mv_ms,
                                      "kernels_ms_per_step": {k: v[0] / args.steps
                                                              for k, v in results["mv"][1].items()}}})
    print(json.dumps(line))
    das.close()
    mvp.close()
    ctx.close()


def run_queue(args) -> None:
    """Mixed probe geometries in one persistent launch: 4 linear frames (128
    elements, 75 plane waves, 512 x 1024, DAS) and 4 phased-array sector
    frames (64 elements, 31 diverging waves, 256 x 1024, DAS), beamformed by
    usx_cu_bf_execute_queue in one launch per step, with the same 8 frames as
    one launch per frame (each plan's autotuned shape) timed beside it."""
    import torch
    import usx
    from usx import capi
    torch.cuda.set_device(0)
    ctx = capi.Context(0)
    _, probe, medium, acq, sim, txs, ph, grid = workload_setup()
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    ch_iq = _capi_channel(capi, probe, medium, acq, txs, is_iq=True, fdem=F0)
    d_sc = torch.from_numpy(_scatterers(ph)).cuda()
    rf = torch.empty((N_TX, N_EL, N_SMP), device="cuda")
    lin_iq = torch.empty((N_TX, N_EL, N_SMP), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.simulate(ch_rf, capi.sim_config(), d_sc.data_ptr(), d_sc.shape[0], None, rf.data_ptr())
    ctx.demodulate(ch_rf, capi.demod_config(), rf.data_ptr(), lin_iq.data_ptr())
    sprobe = usx.Probe()
    sprobe.n_elements, sprobe.pitch, sprobe.element_width = 64, 200e-6, 180e-6
    sprobe.center_frequency, sprobe.bandwidth = 2.5e6, 0.6
    sacq = usx.presets.acquisition(sprobe, depth=0.082, medium=medium, samples_per_wavelength=4.0)
    ssim = usx.Simulator(sprobe, medium, sacq, usx.SimulatorConfig())
    stxs = ssim.make_diverging_waves(usx.angles_deg(-45, 45, 31), 0.01)
    sph = usx.Phantom.speckle_box(-0.06, 0.06, 0.004, 0.084, 0.0, 100_000, 2027)
    sch_rf = _capi_channel(capi, sprobe, medium, sacq, stxs)
    sch_iq = _capi_channel(capi, sprobe, medium, sacq, stxs, is_iq=True, fdem=2.5e6)
    d_ssc = torch.from_numpy(_scatterers(sph)).cuda()
    srf = torch.empty((31, 64, sacq.n_samples), device="cuda")
    sec_iq = torch.empty((31, 64, sacq.n_samples), dtype=torch.complex64, device="cuda")
    ctx.simulate(sch_rf, capi.sim_config(), d_ssc.data_ptr(), d_ssc.shape[0], None, srf.data_ptr())
    ctx.demodulate(sch_rf, capi.demod_config(), srf.data_ptr(), sec_iq.data_ptr())
    del rf, srf
    sgrid = usx.ScanGrid.sector(float(np.deg2rad(-45.0)), float(np.deg2rad(45.0)), 256, 0.005, 0.08, 1024,
                                usx.Vec3(0.0, 0.0, 0.0))
    lin = ctx.plan(ch_iq, capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1),
                                    np.asarray(grid.points).reshape(-1, 3)), capi.bf_config(f_number=1.5))
    sec = ctx.plan(sch_iq, capi.Grid(1, np.asarray(sgrid.axis0), np.asarray(sgrid.axis1),
                                     np.asarray(sgrid.points).reshape(-1, 3)), capi.bf_config(f_number=1.5))
    lin_out = [torch.empty((N0, N1), dtype=torch.complex64, device="cuda") for _ in range(4)]
    sec_out = [torch.empty((256, 1024), dtype=torch.complex64, device="cuda") for _ in range(4)]
    lin.autotune(lin_iq.data_ptr(), lin_out[0].data_ptr(), repeats=1)
    sec.autotune(sec_iq.data_ptr(), sec_out[0].data_ptr(), repeats=1)
    plans = [lin, sec] * 4
    data = [lin_iq.data_ptr(), sec_iq.data_ptr()] * 4
    outs = [o.data_ptr() for pair in zip(lin_out, sec_out) for o in pair]

    def separate():
        for p_, d_, o_ in zip(plans, data, outs):
            p_.execute(d_, o_)

    def queued():
        ctx.execute_queue(plans, data, outs)

    stream = torch.cuda.ExternalStream(ctx.stream())
    for _ in range(args.warmup):
        separate()
        queued()
    ctx.synchronize()
    sep_ms = timed(stream, separate, args.steps)
    capi.profile(ctx, True)
    capi.profile_reset(ctx)
    with ClockSampler(0) as clocks:
        ms = timed(stream, queued, args.steps)
    prof = capi.profile_read(ctx)
    capi.profile(ctx, False)
    per = {k: v[0] / args.steps for k, v in prof.items()}
    line = _stage_line("mixed-probe frames/s in one persistent launch (4 x 128-el 75-PW 512x1024 + 4 x 64-el "
                       "31-DW sector 256x1024, DAS)", "frames/s", 8 * args.steps / (ms / 1e3), args, ms, prof,
                       clocks, {"workload": "queue_4x_linear_512x1024_4x_sector_256x1024", "frames_per_step": 8,
                                "launch": "one das_csum_queue_kernel per step (IQ)"},
                       {"kernel": "das_csum_queue_kernel", "bound": None, "achieved": None, "peak": None, "unit": None,
                        "frac": None, "traffic": None},
                       {"one_launch_per_frame": {"value": 8 * args.steps / (sep_ms / 1e3), "unit": "frames/s",
                                                 "ms_per_step": sep_ms / args.steps},
                        "kernels_ms_per_step": per})
    print(json.dumps(line))
    lin.close()
    sec.close()
    ctx.close()


def run_mixed(args) -> None:
    """Mixed-probe streaming: per step one 128-element linear frame (75 plane
    waves, 512 x 1024) and one 64-element phased-array sector frame (31
    diverging waves, 256 x 1024, L = 32, then envelope, log compression and
    scan conversion to 800 x 800), both by learned MV with the plain-MV
    fallback (the shipped network and gate), captured once into a single CUDA
    graph that each step replays (one launch for the whole mixed batch). The
    sector frame's distance from plain tensor-core MV and both frames'
    fallback rates are reported from one direct execution."""
    import torch
    import usx
    from usx import capi, learned
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    ctx = capi.Context(0, stream=stream.cuda_stream)
    # Linear: the headline acquisition.
    usx_, probe, medium, acq, sim, txs, ph, grid = workload_setup()
    sc = _scatterers(ph)
    ch_rf = _capi_channel(capi, probe, medium, acq, txs)
    ch_iq = _capi_channel(capi, probe, medium, acq, txs, is_iq=True, fdem=F0)
    d_sc = torch.from_numpy(sc).cuda()
    rf = torch.empty((N_TX, N_EL, N_SMP), device="cuda")
    iq_lin = torch.empty((N_TX, N_EL, N_SMP), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.simulate(ch_rf, capi.sim_config(), d_sc.data_ptr(), len(sc), None, rf.data_ptr())
    ctx.demodulate(ch_rf, capi.demod_config(), rf.data_ptr(), iq_lin.data_ptr())
    ctx.synchronize()
    del rf, d_sc
    pts = np.asarray(grid.points).reshape(-1, 3)
    cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), pts)
    mlp = learned.load_mlp(ctx, WEIGHTS)
    lin = ctx.plan(ch_iq, cgrid, capi.bf_config(**LEARNED_KW))
    lin.set_learned(mlp, learned.trained_gate(WEIGHTS))
    lin.set_learned_refine(learned.trained_refine(WEIGHTS))
    lin.set_learned_subspace(True, learned.trained_share_gate(WEIGHTS))
    lin.set_learned_level_gate(learned.trained_level_gate(WEIGHTS))
    lin.set_learned_level_window(*learned.trained_level_window(WEIGHTS))
    f_lin = torch.empty((N0, N1), dtype=torch.complex64, device="cuda")
    lin.autotune(iq_lin.data_ptr(), f_lin.data_ptr(), repeats=1)
    # Sector: 64-element phased array.
    sp = usx.Probe()
    sp.n_elements, sp.pitch, sp.element_width, sp.center_frequency, sp.bandwidth = 64, 200e-6, 180e-6, 2.5e6, 0.6
    sacq = usx.presets.acquisition(sp, depth=0.082, medium=medium, samples_per_wavelength=4.0)
    ssim = usx.Simulator(sp, medium, sacq, usx.SimulatorConfig())
    stx = ssim.make_diverging_waves(usx.angles_deg(-45, 45, 31), 0.01)
    sph = usx.Phantom.speckle_box(-0.06, 0.06, 0.004, 0.084, 0.0, 100_000, 2027)
    ssc = _scatterers(sph)
    sch_rf = _capi_channel(capi, sp, medium, sacq, stx)
    sch_iq = _capi_channel(capi, sp, medium, sacq, stx, is_iq=True, fdem=sp.center_frequency)
    d_ssc = torch.from_numpy(ssc).cuda()
    srf = torch.empty((len(stx), 64, sacq.n_samples), device="cuda")
    iq_sec = torch.empty((len(stx), 64, sacq.n_samples), dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    ctx.simulate(sch_rf, capi.sim_config(), d_ssc.data_ptr(), len(ssc), None, srf.data_ptr())
    ctx.demodulate(sch_rf, capi.demod_config(), srf.data_ptr(), iq_sec.data_ptr())
    ctx.synchronize()
    sgrid = usx.ScanGrid.sector(float(np.deg2rad(-45.0)), float(np.deg2rad(45.0)), 256, 0.005, 0.08, 1024,
                                usx.Vec3(0.0, 0.0, 0.0))
    scg = capi.Grid(1, np.asarray(sgrid.axis0), np.asarray(sgrid.axis1), np.asarray(sgrid.points).reshape(-1, 3))
    sector_mv = dict(f_number=1.5, mv_subarray=32, mv_diagonal_loading=0.01, mv_range_average=2)
    f_sec = torch.empty((256, 1024), dtype=torch.complex64, device="cuda")
    plain = ctx.plan(sch_iq, scg, capi.bf_config(combiner=2, **sector_mv))
    plain.set_mv_mode(args.mv_mode)
    plain.execute(iq_sec.data_ptr(), f_sec.data_ptr())
    ctx.synchronize()                    # the plan ran on the context's stream
    f_sec_plain = f_sec.clone()
    torch.cuda.synchronize()
    plain.close()
    sec = ctx.plan(sch_iq, scg, capi.bf_config(combiner=learned.COMB_LEARNED_MV, **sector_mv))
    sec.set_learned(mlp, learned.trained_gate(WEIGHTS))
    sec.set_learned_refine(learned.trained_refine(WEIGHTS))
    sec.set_learned_subspace(True, learned.trained_share_gate(WEIGHTS))
    sec.set_learned_level_gate(learned.trained_level_gate(WEIGHTS))
    sec.set_learned_level_window(*learned.trained_level_window(WEIGHTS))
    sec.autotune(iq_sec.data_ptr(), f_sec.data_ptr(), repeats=1)
    env, logi = torch.empty((256, 1024), device="cuda"), torch.empty((256, 1024), device="cuda")
    img = torch.empty((800, 800), device="cuda")

    def batch():
        lin.execute(iq_lin.data_ptr(), f_lin.data_ptr())
        sec.execute(iq_sec.data_ptr(), f_sec.data_ptr())
        ctx.envelope(f_sec.data_ptr(), 256, 1024, sp.center_frequency, env.data_ptr())
        ctx.log_compress(env.data_ptr(), 256 * 1024, 60.0, 0.0, -1.0, logi.data_ptr())
        ctx.scan_convert(logi.data_ptr(), scg, 800, 800, 0.0, img.data_ptr())

    with torch.cuda.stream(stream):
        batch()
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            batch()
    with torch.cuda.stream(stream):   # replays run on the stream the events are recorded on
        for _ in range(args.warmup):
            graph.replay()
        stream.synchronize()
        with ClockSampler(0) as clocks:
            ms = timed(stream, graph.replay, args.steps)
        ms_direct = timed(stream, batch, args.steps)
        stream.synchronize()
        # Fallback rates from one direct execution (graph replays bypass the
        # plans' host-side pixel counters).
        lin.learned_stats()
        sec.learned_stats()
        batch()
        stream.synchronize()
        g_lin, p_lin = lin.learned_stats()
        g_sec, p_sec = sec.learned_stats()
        # Per-kernel device times of each frame type from one profiled direct pass.
        profs = {}
        for name, fn in (("linear", lambda: lin.execute(iq_lin.data_ptr(), f_lin.data_ptr())),
                         ("sector", lambda: (sec.execute(iq_sec.data_ptr(), f_sec.data_ptr()),
                                             ctx.envelope(f_sec.data_ptr(), 256, 1024, sp.center_frequency,
                                                          env.data_ptr()),
                                             ctx.log_compress(env.data_ptr(), 256 * 1024, 60.0, 0.0, -1.0,
                                                              logi.data_ptr()),
                                             ctx.scan_convert(logi.data_ptr(), scg, 800, 800, 0.0,
                                                              img.data_ptr())))):
            capi.profile(ctx, True)
            capi.profile_reset(ctx)
            fn()
            stream.synchronize()
            profs[name] = capi.profile_read(ctx)
            capi.profile(ctx, False)
    peaks = load_peaks()
    roof = kernel_roofline(profs["linear"], 1, pts, txs, probe, peaks, learned.trained_refine(WEIGHTS))
    roof["sector_kernels_ms_per_frame"] = {k: v[0] for k, v in profs["sector"].items()}
    launches = sum(v[1] for p in profs.values() for v in p.values()) * args.steps
    torch.cuda.synchronize()
    rel_sec = float((f_sec - f_sec_plain).abs().pow(2).sum().sqrt() / f_sec_plain.abs().pow(2).sum().sqrt())
    line = {"metric": "mixed-batch frames/s (128-el linear 512x1024 + 64-el sector 256x1024 -> 800x800, both "
                      "learned MV with plain-MV fallback)",
            "value": 2 * args.steps / (ms / 1e3), "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (GPU-simulated phantoms)",
            "config": {"workload": "mixed_linear_learned_512x1024_sector_learned_256x1024", "frames_per_step": 2,
                       "launch": "one CUDA graph per step", "sector_mv": sector_mv},
            "direct_launch_ms_per_step": ms_direct / args.steps, "clocks": clocks.summary(),
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": None, "e2e": None,
            "fallback_rate": {"linear": g_lin / max(1, p_lin), "sector": g_sec / max(1, p_sec)},
            "sector_rel_l2_vs_plain_mv": rel_sec}
    print(json.dumps(line))
    lin.close()
    sec.close()
    mlp.close()
    ctx.close()


def run_e2e(usx, grid, raw, rf_host, args, world, learned=None):
    """The same frame through the public API with host buffers: RF up, frame back.
    `learned` = (gate, refine beams, share gate) of the device-timed plan."""
    import torch
    pcfg = usx.PipelineConfig()
    b = pcfg.beamformer
    b.mv_solver = (usx.MvSolver.EXACT if args.workload == "mv_exact" else
                   {1: usx.MvSolver.TENSOR, 2: usx.MvSolver.TENSOR, 3: usx.MvSolver.FP32}[args.mv_mode])
    if learned is not None:
        b.learned_gate, b.learned_refine, b.learned_share_gate, b.learned_level_gate = learned
    kw = WORKLOADS[args.workload]
    b.f_number = kw["f_number"]
    b.combiner = usx.Combiner(kw.get("combiner", 0))
    b.coherence_factor = bool(kw.get("coherence_factor", 0))
    b.mv_subarray = kw.get("mv_subarray", 16)
    b.mv_diagonal_loading = kw.get("mv_diagonal_loading", 0.01)
    b.mv_range_average = kw.get("mv_range_average", 2)
    pcfg.beamformer = b
    pipe = usx.ImagingPipeline(grid, pcfg)
    # Warm-up as for the device-timed loop: the first call builds and tunes the
    # plan, the next still pays first-touch costs of the host buffers.
    for _ in range(max(3, args.warmup)):
        pipe.process_frame(raw)
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        pipe.process_frame(raw)
    e2e_s = (time.perf_counter() - t) / e2e_steps
    return {"value": world / e2e_s, "unit": "frames/s", "h2d_bytes_per_step": int(rf_host.nbytes),
            "d2h_bytes_per_step": int(N0 * N1 * 8), "api": "usx.ImagingPipeline.process_frame(RF ChannelData)"}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="learned",
                    choices=sorted(WORKLOADS) + ["simulate", "demod", "doppler", "strain", "post", "batch", "sector", "queue",
                                                   "mixed"])
    ap.add_argument("--scatterers", type=int, default=100_000, help="simulate workload: phantom size")
    ap.add_argument("--gate", type=float, default=None, help="learned workload: gate (default: the weights' report)")
    ap.add_argument("--refine", type=int, default=None, help="learned workload: subspace beams (default: report)")
    ap.add_argument("--share-gate", type=float, default=None,
                    help="learned workload: gate on the network direction's share (default: report)")
    ap.add_argument("--level-gate", type=float, default=None,
                    help="learned workload: gate on tr(R) over its depth's level (default: report)")
    ap.add_argument("--lines", type=int, default=N0, help="lateral lines timed (profiling cases use fewer)")
    ap.add_argument("--mv-mode", type=int, default=3, choices=[1, 2, 3],
                    help="plain MV solver (mv workload, the headline's plain MV and the learned plan's gated "
                         "pixels): 1 tcgen05 BF16 covariance + refinement, 2 the same on mma.sync, "
                         "3 FP32 lag-recurrence covariance")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-two-streams", dest="two_streams", action="store_false",
                    help="learned workload: skip the two-frames-in-flight timing (two plans on two streams)")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("simulate", "demod"):
        run_stage(args)
    elif args.workload == "doppler":
        run_doppler(args)
    elif args.workload == "strain":
        run_strain(args)
    elif args.workload == "post":
        run_post(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "sector":
        run_sector(args)
    elif args.workload == "queue":
        run_queue(args)
    elif args.workload == "mixed":
        run_mixed(args)
    else:
        run_ours(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
