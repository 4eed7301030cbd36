"""ctypes binding of the C-ABI in include/usx_cu.h (libusx_cu.so).

This is the device-resident door into the kernels: every data argument is a
device address (an int, e.g. `torch.Tensor.data_ptr()`), descriptors are
ctypes structures mirroring include/usx_types.h, and each call maps a non-zero
status to an exception (ValueError for USX_ERR_INVALID, as the reference maps
std::invalid_argument; RuntimeError otherwise). It is also the template for a
binding from another language: every call here is one C function.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parents[2] / "lib" / "libusx_cu.so"

USX_OK, USX_ERR_INVALID = 0, 1

f32p = C.POINTER(C.c_float)
vp = C.c_void_p


class Probe(C.Structure):
    _fields_ = [("n_elements", C.c_int32), ("pitch", C.c_float), ("element_width", C.c_float),
                ("elevation_height", C.c_float), ("center_frequency", C.c_float), ("bandwidth", C.c_float)]


class Medium(C.Structure):
    _fields_ = [("speed_of_sound", C.c_float), ("attenuation", C.c_float), ("density", C.c_float)]


class Acquisition(C.Structure):
    _fields_ = [("sampling_frequency", C.c_float), ("n_samples", C.c_int32), ("t0", C.c_float), ("prf", C.c_float)]


class Transmit(C.Structure):
    _fields_ = [("type", C.c_int32), ("angle", C.c_float), ("focus", C.c_float * 3), ("origin", C.c_float * 3),
                ("delays", f32p), ("apodization", f32p)]


class ChannelDesc(C.Structure):
    _fields_ = [("probe", Probe), ("medium", Medium), ("acq", Acquisition), ("n_events", C.c_int32),
                ("transmits", C.POINTER(Transmit)), ("is_iq", C.c_int32), ("demodulation_frequency", C.c_float)]


class GridDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("n_axis0", C.c_int32), ("n_axis1", C.c_int32), ("apex", C.c_float * 3),
                ("axis0", f32p), ("axis1", f32p)]


class BeamformerConfig(C.Structure):
    _fields_ = [("f_number", C.c_float), ("rx_window", C.c_int32), ("tukey_alpha", C.c_float),
                ("combiner", C.c_int32), ("compounding", C.c_int32), ("transmit_weighting", C.c_int32),
                ("coherence_factor", C.c_int32), ("mv_subarray", C.c_int32), ("mv_diagonal_loading", C.c_float),
                ("mv_range_average", C.c_int32)]


class DemodConfig(C.Structure):
    _fields_ = [("demodulation_frequency", C.c_float), ("cutoff_fraction", C.c_float),
                ("filter_taps", C.c_int32), ("decimation", C.c_int32)]


class SimulatorConfig(C.Structure):
    _fields_ = [("pulse_cycles", C.c_float), ("tx_window", C.c_int32), ("tx_f_number", C.c_float),
                ("oversampling", C.c_int32), ("full_transmit_diffraction", C.c_int32),
                ("incident_trim_db", C.c_float), ("max_incident_window_us", C.c_float),
                ("apply_attenuation", C.c_int32), ("apply_directivity", C.c_int32),
                ("apply_spreading", C.c_int32), ("noise_db", C.c_float), ("noise_seed", C.c_uint32),
                ("enable_motion", C.c_int32)]


class DopplerConfig(C.Structure):
    _fields_ = [("wall_filter", C.c_int32), ("polynomial_order", C.c_int32), ("loupas", C.c_int32),
                ("kernel_axial", C.c_int32), ("kernel_lateral", C.c_int32), ("power_threshold_db", C.c_float),
                ("coherence_threshold", C.c_float)]


def bf_config(**kw) -> BeamformerConfig:
    d = dict(f_number=1.75, rx_window=1, tukey_alpha=0.5, combiner=0, compounding=0, transmit_weighting=1,
             coherence_factor=0, mv_subarray=16, mv_diagonal_loading=1e-2, mv_range_average=2)
    d.update(kw)
    return BeamformerConfig(**d)


def demod_config(**kw) -> DemodConfig:
    d = dict(demodulation_frequency=0.0, cutoff_fraction=0.5, filter_taps=33, decimation=1)
    d.update(kw)
    return DemodConfig(**d)


def sim_config(**kw) -> SimulatorConfig:
    d = dict(pulse_cycles=2.5, tx_window=1, tx_f_number=2.0, oversampling=4, full_transmit_diffraction=1,
             incident_trim_db=-40.0, max_incident_window_us=30.0, apply_attenuation=1, apply_directivity=1,
             apply_spreading=1, noise_db=-60.0, noise_seed=7, enable_motion=1)
    d.update(kw)
    return SimulatorConfig(**d)


def doppler_config(**kw) -> DopplerConfig:
    d = dict(wall_filter=1, polynomial_order=1, loupas=1, kernel_axial=4, kernel_lateral=1,
             power_threshold_db=-35.0, coherence_threshold=0.35)
    d.update(kw)
    return DopplerConfig(**d)


class Channel:
    """A usx_channel_desc with its transmit arrays kept alive.

    `transmits`: list of dicts with keys type, angle, focus, origin, delays, apodization."""

    def __init__(self, probe: Probe, medium: Medium, acq: Acquisition, transmits, is_iq=False, fdem=0.0):
        n = len(transmits)
        self._arrays = []
        self.tx = (Transmit * max(n, 1))()
        for e, t in enumerate(transmits):
            x = self.tx[e]
            x.type = int(t.get("type", 1))
            x.angle = float(t.get("angle", 0.0))
            for k in range(3):
                x.focus[k] = float(t.get("focus", (0, 0, 0.03))[k])
                x.origin[k] = float(t.get("origin", (0, 0, 0))[k])
            for name, field in (("delays", "delays"), ("apodization", "apodization")):
                arr = t.get(name)
                if arr is None or len(arr) == 0:
                    setattr(x, field, None)
                else:
                    a = np.ascontiguousarray(arr, dtype=np.float32)
                    self._arrays.append(a)
                    setattr(x, field, a.ctypes.data_as(f32p))
        self.desc = ChannelDesc(probe, medium, acq, n, C.cast(self.tx, C.POINTER(Transmit)), int(is_iq), float(fdem))


class Grid:
    """A usx_grid_desc plus its host point list (n_axis0*n_axis1, 3) float32."""

    def __init__(self, gtype, axis0, axis1, points, apex=(0.0, 0.0, 0.0)):
        self.axis0 = np.ascontiguousarray(axis0, dtype=np.float32)
        self.axis1 = np.ascontiguousarray(axis1, dtype=np.float32)
        self.points = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        ap = (C.c_float * 3)(*[float(v) for v in apex])
        self.desc = GridDesc(int(gtype), len(self.axis0), len(self.axis1), ap,
                             self.axis0.ctypes.data_as(f32p), self.axis1.ctypes.data_as(f32p))

    @property
    def shape(self):
        return (len(self.axis0), len(self.axis1))


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run ultrasound-engine_gb300/build.py")
        _lib = C.CDLL(str(LIB_PATH))
        _lib.usx_cu_last_error.restype = C.c_char_p
        _lib.usx_cu_ctx_stream.restype = vp
    return _lib


def check(rc: int, what: str) -> None:
    if rc == USX_OK:
        return
    msg = lib().usx_cu_last_error().decode()
    if rc == USX_ERR_INVALID:
        raise ValueError(f"{what}: {msg}")
    raise RuntimeError(f"{what} failed ({rc}): {msg}")


CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy: the stream torch calls "default" (handle 0)


class Context:
    """usx_ctx on one device.

    stream=None: the context creates its own non-blocking stream (callers must
    order their own copies against it, e.g. with synchronize()).
    stream=int: the context adopts that cudaStream_t; 0 (torch's default
    stream) means the legacy default stream, so work is ordered with torch's."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._h = vp()
        if stream is not None and stream == 0:
            stream = CUDA_STREAM_LEGACY
        check(lib().usx_cu_ctx_create(int(device), vp(stream) if stream else None, C.byref(self._h)),
              "usx_cu_ctx_create")

    @property
    def handle(self):
        return self._h

    def stream(self) -> int:
        return lib().usx_cu_ctx_stream(self._h) or 0

    def synchronize(self):
        check(lib().usx_cu_synchronize(self._h), "synchronize")

    def close(self):
        if self._h:
            lib().usx_cu_ctx_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------- kernels
    def simulate(self, ch: Channel, cfg: SimulatorConfig, scat_ptr: int, n_scat: int, noise_ptr: int | None,
                 rf_ptr: int, want_stats: bool = False):
        stats = (C.c_double * 2)()
        check(lib().usx_cu_simulate(self._h, C.byref(ch.desc), C.byref(cfg), vp(scat_ptr), C.c_int64(n_scat),
                                    vp(noise_ptr) if noise_ptr else None, vp(rf_ptr),
                                    stats if want_stats else None), "simulate")
        return (stats[0], stats[1]) if want_stats else None

    def demodulate(self, ch: Channel, cfg: DemodConfig, rf_ptr: int, iq_ptr: int) -> float:
        f = C.c_float()
        check(lib().usx_cu_demodulate(self._h, C.byref(ch.desc), C.byref(cfg), vp(rf_ptr), vp(iq_ptr),
                                      C.byref(f)), "demodulate")
        return f.value

    def plan(self, ch: Channel, grid: Grid, cfg: BeamformerConfig, ev_begin=0, ev_end=-1) -> "Plan":
        return Plan(self, ch, grid, cfg, ev_begin, ev_end)

    def envelope(self, frame_ptr, n0, n1, fdem, env_ptr):
        check(lib().usx_cu_envelope(self._h, vp(frame_ptr), n0, n1, C.c_float(fdem), vp(env_ptr)), "envelope")

    def apply_tgc(self, env_ptr, n0, n1, points_ptr, atten, f0, out_ptr):
        check(lib().usx_cu_apply_tgc(self._h, vp(env_ptr), n0, n1, vp(points_ptr), C.c_float(atten),
                                     C.c_float(f0), vp(out_ptr)), "apply_tgc")

    def log_compress(self, env_ptr, n, dr, gain, ref, out_ptr):
        check(lib().usx_cu_log_compress(self._h, vp(env_ptr), C.c_int64(n), C.c_float(dr), C.c_float(gain),
                                        C.c_float(ref), vp(out_ptr)), "log_compress")

    def scan_convert(self, img_ptr, grid: Grid, width, height, fill, px_ptr):
        ext = (C.c_float * 4)()
        check(lib().usx_cu_scan_convert(self._h, vp(img_ptr), C.byref(grid.desc), grid.points.ctypes.data_as(f32p),
                                        width, height, C.c_float(fill), vp(px_ptr), ext), "scan_convert")
        return np.array(ext[:], np.float32)

    def wall_filter(self, ens_ptr, n_frames, n_pix, wtype, order, out_ptr):
        check(lib().usx_cu_wall_filter(self._h, vp(ens_ptr), n_frames, C.c_int64(n_pix), wtype, order,
                                       vp(out_ptr)), "wall_filter")

    def power_doppler(self, ens_ptr, n_frames, n_pix, wtype, order, out_ptr):
        check(lib().usx_cu_power_doppler(self._h, vp(ens_ptr), n_frames, C.c_int64(n_pix), wtype, order,
                                         vp(out_ptr)), "power_doppler")

    def color_flow(self, ens_ptr, n_frames, n0, n1, axis1, fdem, prf, c, cfg: DopplerConfig, vel, pw, var, valid):
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        nyq = C.c_float()
        check(lib().usx_cu_color_flow(self._h, vp(ens_ptr), n_frames, n0, n1, ax.ctypes.data_as(f32p),
                                      C.c_float(fdem), C.c_float(prf), C.c_float(c), C.byref(cfg), vp(vel), vp(pw),
                                      vp(var), vp(valid), C.byref(nyq)), "color_flow")
        return nyq.value

    def color_flow_batch(self, ens_ptr, n_frames, frame_offset, n0, n1, axis1, fdem, prf, c,
                         cfg: DopplerConfig, vel, pw, var, valid):
        nf = np.ascontiguousarray(n_frames, dtype=np.int32)
        off = np.ascontiguousarray(frame_offset, dtype=np.int64)
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        check(lib().usx_cu_color_flow_batch(self._h, vp(ens_ptr), len(nf), nf.ctypes.data_as(C.POINTER(C.c_int)),
                                            off.ctypes.data_as(C.POINTER(C.c_int64)), n0, n1,
                                            ax.ctypes.data_as(f32p), C.c_float(fdem), C.c_float(prf), C.c_float(c),
                                            C.byref(cfg), vp(vel), vp(pw), vp(var), vp(valid)),
              "color_flow_batch")

    def execute_queue(self, plans, data_ptrs, frame_ptrs) -> None:
        """One frame per (plan, data, frame) entry, all in one persistent launch."""
        n = len(plans)
        P = (vp * n)(*[p._h for p in plans])
        D = (vp * n)(*[vp(x) for x in data_ptrs])
        F = (vp * n)(*[vp(x) for x in frame_ptrs])
        check(lib().usx_cu_bf_execute_queue(self._h, n, P, D, F), "bf_execute_queue")

    def axial_displacement(self, a_ptr, b_ptr, n0, n1, axis1, fdem, c, ka, kl, max_lag, axial_ptr, corr_ptr):
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        check(lib().usx_cu_axial_displacement(self._h, vp(a_ptr), vp(b_ptr), n0, n1, ax.ctypes.data_as(f32p),
                                              C.c_float(fdem), C.c_float(c), ka, kl, max_lag, vp(axial_ptr),
                                              vp(corr_ptr)), "axial_displacement")

    def axial_strain(self, axial_ptr, n0, n1, axis1, fit, out_ptr):
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        check(lib().usx_cu_axial_strain(self._h, vp(axial_ptr), n0, n1, ax.ctypes.data_as(f32p), fit,
                                        vp(out_ptr)), "axial_strain")


class Plan:
    """usx_bf_plan: a frozen beamforming configuration on the device."""

    def __init__(self, ctx: Context, ch: Channel, grid: Grid, cfg: BeamformerConfig, ev_begin=0, ev_end=-1):
        self.ctx = ctx
        self._h = vp()
        self._keep = (ch, grid, cfg)
        check(lib().usx_cu_bf_plan_create(ctx.handle, C.byref(ch.desc), C.byref(grid.desc),
                                          grid.points.ctypes.data_as(f32p), C.byref(cfg), ev_begin, ev_end,
                                          C.byref(self._h)), "bf_plan_create")

    def execute(self, data_ptr: int, frame_ptr: int):
        check(lib().usx_cu_bf_execute(self._h, vp(data_ptr), vp(frame_ptr)), "bf_execute")

    def execute_batch(self, n_frames, data_ptr, data_stride, frames_ptr, frame_stride):
        check(lib().usx_cu_bf_execute_batch(self._h, n_frames, vp(data_ptr), C.c_int64(data_stride),
                                            vp(frames_ptr), C.c_int64(frame_stride)), "bf_execute_batch")

    def execute_sequence(self, events_per_frame, n_frames, data_ptr, frames_ptr, frame_stride):
        check(lib().usx_cu_bf_execute_sequence(self._h, events_per_frame, n_frames, vp(data_ptr), vp(frames_ptr),
                                               C.c_int64(frame_stride)), "bf_execute_sequence")

    def set_precision(self, precision: int) -> None:
        """0: fast (default); 1: every operation in the reference's order."""
        check(lib().usx_cu_bf_plan_set_precision(self._h, int(precision)), "bf_plan_set_precision")

    def set_mv_mode(self, mode: int) -> None:
        """0: FP32 in the reference's order; 1: BF16 covariance on tcgen05 + refinement;
        2: the same with the covariance on warp-level mma.sync; 3: FP32 covariance by
        the lag recurrence in the solve kernel, one FP32 solve."""
        check(lib().usx_cu_bf_plan_set_mv_mode(self._h, int(mode)), "bf_plan_set_mv_mode")

    def mv_stats(self):
        a, b = C.c_int64(), C.c_int64()
        check(lib().usx_cu_bf_plan_mv_stats(self._h, C.byref(a), C.byref(b)), "bf_plan_mv_stats")
        return a.value, b.value

    def set_learned(self, mlp: "Mlp | None", gate: float = 0.05) -> None:
        """Attach the network of a LEARNED_MV plan (kept alive by the plan)."""
        check(lib().usx_cu_bf_plan_set_learned(self._h, mlp.handle if mlp else None, C.c_float(gate)),
              "bf_plan_set_learned")
        self._mlp = mlp

    def autotune(self, data_ptr: int, frame_ptr: int, repeats: int = 2):
        """Time every delay-and-sum variant on this acquisition, keep the
        fastest; returns (chosen index, [ms per variant])."""
        n = lib().usx_cu_bf_variant_count()
        ms = (C.c_float * n)()
        check(lib().usx_cu_bf_plan_autotune(self._h, vp(data_ptr), vp(frame_ptr), int(repeats), ms),
              "bf_plan_autotune")
        return self.variant(), list(ms)

    def variant(self) -> int:
        v = C.c_int()
        check(lib().usx_cu_bf_plan_get_variant(self._h, C.byref(v)), "bf_plan_get_variant")
        return v.value

    def set_variant(self, index: int) -> None:
        check(lib().usx_cu_bf_plan_set_variant(self._h, int(index)), "bf_plan_set_variant")

    def set_learned_refine(self, n_beams: int) -> None:
        """Negative: the network's weights as predicted; 0, 2, 4, 6: exact Capon
        solve within span{1, network weights, n_beams DFT beams}."""
        check(lib().usx_cu_bf_plan_set_learned_refine(self._h, int(n_beams)), "bf_plan_set_learned_refine")

    def set_learned_subspace(self, use_network: bool = True, max_network_share: float = float("inf")) -> None:
        """The refinement's basis with or without the network's direction, and
        the gate on the share of the output-power reduction that direction
        carries (pixels above it go to the exact solver)."""
        check(lib().usx_cu_bf_plan_set_learned_subspace(self._h, int(bool(use_network)),
                                                         C.c_float(max_network_share)),
              "bf_plan_set_learned_subspace")

    def set_learned_level_gate(self, max_level_ratio: float = float("inf")) -> None:
        """Pixels whose covariance trace exceeds this multiple of their depth's
        geometric-mean trace go to the exact solver (+inf: off)."""
        check(lib().usx_cu_bf_plan_set_learned_level_gate(self._h, C.c_float(max_level_ratio)),
              "bf_plan_set_learned_level_gate")

    def set_learned_level_window(self, half_lines: int = 0, half_depths: int = 0) -> None:
        """The level gate's neighbourhood (+/- lines, +/- depths): a pixel goes to
        the exact solver when any pixel of it is above its depth's level."""
        check(lib().usx_cu_bf_plan_set_learned_level_window(self._h, int(half_lines), int(half_depths)),
              "bf_plan_set_learned_level_window")

    def learned_stats(self):
        """(pixels gated to the exact solver, pixels beamformed) since the last call."""
        a, b = C.c_int64(), C.c_int64()
        check(lib().usx_cu_bf_plan_learned_stats(self._h, C.byref(a), C.byref(b)), "bf_plan_learned_stats")
        return a.value, b.value

    def set_training_export(self, features_ptr: int | None, weights_ptr: int | None, valid_ptr: int | None):
        """Per-pixel features [rows][256], Capon weights [rows][128] and valid
        flags [rows] (device pointers) written by every execution; None turns it off."""
        check(lib().usx_cu_bf_plan_set_training_export(self._h, vp(features_ptr) if features_ptr else None,
                                                       vp(weights_ptr) if weights_ptr else None,
                                                       vp(valid_ptr) if valid_ptr else None),
              "bf_plan_set_training_export")

    def workspace_bytes(self) -> int:
        n = C.c_size_t()
        check(lib().usx_cu_bf_plan_workspace(self._h, C.byref(n)), "bf_plan_workspace")
        return n.value

    def close(self):
        if self._h:
            lib().usx_cu_bf_plan_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mlp:
    """usx_mlp: fully connected ReLU network trained and run on the device
    (BF16 GEMMs with FP32 accumulation, FP32 master weights, Adam)."""

    def __init__(self, ctx: Context, dims, seed: int = 0):
        self.ctx = ctx
        self.dims = [int(d) for d in dims]
        self._h = vp()
        arr = (C.c_int * len(self.dims))(*self.dims)
        check(lib().usx_cu_mlp_create(ctx.handle, len(self.dims) - 1, arr, C.c_uint64(seed), C.byref(self._h)),
              "mlp_create")

    @property
    def handle(self):
        return self._h

    @property
    def n_params(self) -> int:
        n = C.c_int64()
        check(lib().usx_cu_mlp_num_params(self._h, C.byref(n)), "mlp_num_params")
        return n.value

    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        check(lib().usx_cu_mlp_get_params(self._h, out.ctypes.data_as(f32p)), "mlp_get_params")
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {p.size}")
        check(lib().usx_cu_mlp_set_params(self._h, p.ctypes.data_as(f32p)), "mlp_set_params")

    def layers(self, params=None):
        """[(W [din, dout], b [dout]), ...] views of a parameter vector."""
        p = self.get_params() if params is None else params
        out, o = [], 0
        for din, dout in zip(self.dims[:-1], self.dims[1:]):
            w = p[o:o + din * dout].reshape(din, dout)
            o += din * dout
            b = p[o:o + dout]
            o += dout
            out.append((w, b))
        return out

    LOSS_MSE, LOSS_LMV_OUTPUT, LOSS_LMV_SUBSPACE = 0, 1, 2

    def set_loss(self, kind: int, beta: float = 0.0) -> None:
        """Training loss: LOSS_MSE (masked MSE) or LOSS_LMV_OUTPUT (learned-MV
        combiner output error + beta * weight MSE)."""
        check(lib().usx_cu_mlp_set_loss(self._h, int(kind), C.c_float(beta)), "mlp_set_loss")

    GEMM_AUTO, GEMM_MMA_SYNC = 0, 1

    def set_gemm_path(self, path: int) -> None:
        """Forward GEMM: GEMM_AUTO (tcgen05 wherever the layer shape allows)
        or GEMM_MMA_SYNC (the mma.sync GEMM for every layer)."""
        check(lib().usx_cu_mlp_set_gemm_path(self._h, int(path)), "mlp_set_gemm_path")

    def forward(self, x_ptr: int, rows: int, y_ptr: int) -> None:
        check(lib().usx_cu_mlp_forward(self._h, vp(x_ptr), C.c_int64(rows), vp(y_ptr)), "mlp_forward")

    def train_step(self, x_ptr: int, t_ptr: int, mask_ptr: int | None, rows: int, lr: float,
                   want_loss: bool = False, want_grad: bool = False):
        """One step; returns (loss or None, gradient vector or None)."""
        loss = C.c_float()
        grad = np.empty(self.n_params, np.float32) if want_grad else None
        check(lib().usx_cu_mlp_train_step(self._h, vp(x_ptr), vp(t_ptr), vp(mask_ptr) if mask_ptr else None,
                                          C.c_int64(rows), C.c_float(lr),
                                          C.byref(loss) if want_loss else None,
                                          grad.ctypes.data_as(f32p) if want_grad else None), "mlp_train_step")
        return (loss.value if want_loss else None), grad

    def close(self):
        if self._h:
            lib().usx_cu_mlp_destroy(self._h)
            self._h = vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def das_variants() -> list:
    """(channel group, tile lines, min resident CTAs, lines per warp, deepest
    tiles first, kind) of each delay-and-sum variant; kind 0: thread per
    pixel, 1: staged trace windows, 2: transmit table, 3: producer-warp ring,
    4: channel warps with a per-pixel transmit table (tile lines = pixel
    warps)."""
    out = []
    for i in range(lib().usx_cu_bf_variant_count()):
        g, t, m, w, d, k = C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib().usx_cu_bf_variant_info(i, C.byref(g), C.byref(t), C.byref(m), C.byref(w)), "bf_variant_info")
        check(lib().usx_cu_bf_variant_order(i, C.byref(d)), "bf_variant_order")
        check(lib().usx_cu_bf_variant_kind(i, C.byref(k)), "bf_variant_kind")
        out.append((g.value, t.value, m.value, w.value, d.value, k.value))
    return out


def profile(ctx: Context, on: bool = True) -> None:
    """Record CUDA events around every launch on ctx's stream."""
    check(lib().usx_cu_profile_enable(ctx.handle, 1 if on else 0), "profile_enable")


def profile_reset(ctx: Context) -> None:
    check(lib().usx_cu_profile_reset(ctx.handle), "profile_reset")


def profile_read(ctx: Context) -> dict:
    """{kernel name: (total device ms, launches)} since the last reset."""
    out = {}
    name = C.create_string_buffer(128)
    ms = C.c_double()
    n = C.c_int64()
    i = 0
    while lib().usx_cu_profile_read(ctx.handle, i, name, 128, C.byref(ms), C.byref(n)) == USX_OK:
        out[name.value.decode()] = (ms.value, n.value)
        i += 1
    return out


def color_flow_noalloc(stream: int, ens_ptr, n_frames, n0, n1, axis1, fdem, prf, c, cfg: DopplerConfig,
                       vel, pw, var, valid) -> float:
    """usx_cu_color_flow_noalloc: colour flow on `stream` (0: legacy default
    stream) with no device allocation, working memory in the library's fixed
    8 MiB array (n_frames * n0 * n1 <= 1048576; larger raises ValueError).
    Calls overlapping on the GPU share that array and must be serialised."""
    ax = np.ascontiguousarray(axis1, dtype=np.float32)
    nyq = C.c_float()
    check(lib().usx_cu_color_flow_noalloc(vp(stream) if stream else None, vp(ens_ptr), n_frames, n0, n1,
                                          ax.ctypes.data_as(f32p), C.c_float(fdem), C.c_float(prf), C.c_float(c),
                                          C.byref(cfg), vp(vel), vp(pw), vp(var), vp(valid), C.byref(nyq)),
          "color_flow_noalloc")
    return nyq.value
