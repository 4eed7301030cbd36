"""ctypes bindings for the CPU oracle (and, where it was built, the reference).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product. `liboracle.so` is the
plain-C restatement in this directory (built by __graft_entry__.build());
`_ref/libusx_ref.so` is the reference engine compiled from its own sources by
build_ref.sh, available only where the reference checkout exists.

The ctypes structures mirror include/usx_types.h field for field.
"""

from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libusx_ref.so"

f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)
u8p = C.POINTER(C.c_ubyte)


class Probe(C.Structure):
    _fields_ = [("n_elements", C.c_int32), ("pitch", C.c_float), ("element_width", C.c_float),
                ("elevation_height", C.c_float), ("center_frequency", C.c_float),
                ("bandwidth", C.c_float)]


class Medium(C.Structure):
    _fields_ = [("speed_of_sound", C.c_float), ("attenuation", C.c_float), ("density", C.c_float)]


class Acquisition(C.Structure):
    _fields_ = [("sampling_frequency", C.c_float), ("n_samples", C.c_int32), ("t0", C.c_float),
                ("prf", C.c_float)]


class Transmit(C.Structure):
    _fields_ = [("type", C.c_int32), ("angle", C.c_float), ("focus", C.c_float * 3),
                ("origin", C.c_float * 3), ("delays", f32p), ("apodization", f32p)]


class ChannelDesc(C.Structure):
    _fields_ = [("probe", Probe), ("medium", Medium), ("acq", Acquisition),
                ("n_events", C.c_int32), ("transmits", C.POINTER(Transmit)),
                ("is_iq", C.c_int32), ("demodulation_frequency", C.c_float)]


class BeamformerConfig(C.Structure):
    _fields_ = [("f_number", C.c_float), ("rx_window", C.c_int32), ("tukey_alpha", C.c_float),
                ("combiner", C.c_int32), ("compounding", C.c_int32),
                ("transmit_weighting", C.c_int32), ("coherence_factor", C.c_int32),
                ("mv_subarray", C.c_int32), ("mv_diagonal_loading", C.c_float),
                ("mv_range_average", C.c_int32)]


class DemodConfig(C.Structure):
    _fields_ = [("demodulation_frequency", C.c_float), ("cutoff_fraction", C.c_float),
                ("filter_taps", C.c_int32), ("decimation", C.c_int32)]


class SimulatorConfig(C.Structure):
    _fields_ = [("pulse_cycles", C.c_float), ("tx_window", C.c_int32), ("tx_f_number", C.c_float),
                ("oversampling", C.c_int32), ("full_transmit_diffraction", C.c_int32),
                ("incident_trim_db", C.c_float), ("max_incident_window_us", C.c_float),
                ("apply_attenuation", C.c_int32), ("apply_directivity", C.c_int32),
                ("apply_spreading", C.c_int32), ("noise_db", C.c_float),
                ("noise_seed", C.c_uint32), ("enable_motion", C.c_int32)]


class DopplerConfig(C.Structure):
    _fields_ = [("wall_filter", C.c_int32), ("polynomial_order", C.c_int32), ("loupas", C.c_int32),
                ("kernel_axial", C.c_int32), ("kernel_lateral", C.c_int32),
                ("power_threshold_db", C.c_float), ("coherence_threshold", C.c_float)]


def probe(n_elements=128, pitch=300e-6, element_width=270e-6, elevation_height=5e-3,
          center_frequency=5e6, bandwidth=0.6) -> Probe:
    return Probe(n_elements, pitch, element_width, elevation_height, center_frequency, bandwidth)


def medium(c=1540.0, attenuation=0.5, density=1000.0) -> Medium:
    return Medium(c, attenuation, density)


def acquisition(fs=40e6, n_samples=2048, t0=0.0, prf=5000.0) -> Acquisition:
    return Acquisition(fs, n_samples, t0, prf)


def bf_config(**kw) -> BeamformerConfig:
    d = dict(f_number=1.75, rx_window=1, tukey_alpha=0.5, combiner=0, compounding=0,
             transmit_weighting=1, coherence_factor=0, mv_subarray=16, mv_diagonal_loading=1e-2,
             mv_range_average=2)
    d.update(kw)
    return BeamformerConfig(**d)


def demod_config(**kw) -> DemodConfig:
    d = dict(demodulation_frequency=0.0, cutoff_fraction=0.5, filter_taps=33, decimation=1)
    d.update(kw)
    return DemodConfig(**d)


def sim_config(**kw) -> SimulatorConfig:
    d = dict(pulse_cycles=2.5, tx_window=1, tx_f_number=2.0, oversampling=4,
             full_transmit_diffraction=1, incident_trim_db=-40.0, max_incident_window_us=30.0,
             apply_attenuation=1, apply_directivity=1, apply_spreading=1, noise_db=-60.0,
             noise_seed=7, enable_motion=1)
    d.update(kw)
    return SimulatorConfig(**d)


def doppler_config(**kw) -> DopplerConfig:
    d = dict(wall_filter=1, polynomial_order=1, loupas=1, kernel_axial=4, kernel_lateral=1,
             power_threshold_db=-35.0, coherence_threshold=0.35)
    d.update(kw)
    return DopplerConfig(**d)


@dataclass
class TxSet:
    """Transmit events with their delay/apodization arrays kept alive."""
    types: np.ndarray
    angles: np.ndarray
    focus: np.ndarray
    origin: np.ndarray
    delays: np.ndarray        # (n_ev, n_el) float32
    apod: np.ndarray          # (n_ev, n_el) float32
    _arr: object = field(default=None, repr=False)

    def __len__(self):
        return len(self.types)

    def ctypes_array(self):
        n = len(self)
        arr = (Transmit * n)()
        self.delays = np.ascontiguousarray(self.delays, dtype=np.float32)
        self.apod = np.ascontiguousarray(self.apod, dtype=np.float32)
        for e in range(n):
            t = arr[e]
            t.type = int(self.types[e])
            t.angle = float(self.angles[e])
            for k in range(3):
                t.focus[k] = float(self.focus[e, k])
                t.origin[k] = float(self.origin[e, k])
            t.delays = self.delays[e].ctypes.data_as(f32p)
            t.apodization = self.apod[e].ctypes.data_as(f32p)
        self._arr = arr
        return arr

    def repeat(self, n):
        return TxSet(np.tile(self.types, n), np.tile(self.angles, n), np.tile(self.focus, (n, 1)),
                     np.tile(self.origin, (n, 1)), np.tile(self.delays, (n, 1)),
                     np.tile(self.apod, (n, 1)))

    def subset(self, idx):
        idx = np.asarray(idx)
        return TxSet(self.types[idx], self.angles[idx], self.focus[idx], self.origin[idx],
                     self.delays[idx], self.apod[idx])


def channel_desc(pr: Probe, med: Medium, acq: Acquisition, txs: TxSet, is_iq=False, fdem=0.0):
    arr = txs.ctypes_array()
    cd = ChannelDesc(pr, med, acq, len(txs), C.cast(arr, C.POINTER(Transmit)), int(is_iq), fdem)
    cd._keep = (arr, txs)
    return cd


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


class Lib:
    """The oracle (`kind='oracle'`) or the reference shim (`kind='ref'`)."""

    def __init__(self, kind: str = "oracle"):
        self.kind = kind
        path = ORACLE_SO if kind == "oracle" else REF_SO
        if not path.exists():
            raise FileNotFoundError(f"{path} not built")
        self.lib = C.CDLL(str(path))

    # --- oracle (C restatement) -------------------------------------------
    def _fn(self, name, prec):
        return getattr(self.lib, f"{name}_{prec}")

    @staticmethod
    def _dt(prec):
        return np.float32 if prec == "f32" else np.float64

    @staticmethod
    def _pt(prec):
        return f32p if prec == "f32" else f64p

    def simulate(self, cd, scfg, scat, noise_z=None, prec="f32"):
        scat = np.ascontiguousarray(scat, dtype=np.float32)
        shape = (cd.n_events, cd.probe.n_elements, cd.acq.n_samples)
        rf = np.zeros(shape, dtype=self._dt(prec))
        z = None if noise_z is None else np.ascontiguousarray(noise_z, dtype=np.float32)
        f = self._fn("orc_simulate", prec)
        f.argtypes = [C.c_void_p, C.c_void_p, f32p, C.c_long, f32p, self._pt(prec)]
        f(C.byref(cd), C.byref(scfg), _ptr(scat, f32p), len(scat),
          None if z is None else _ptr(z, f32p), _ptr(rf, self._pt(prec)))
        return rf

    def demodulate(self, cd, dcfg, rf, prec="f32"):
        dec = max(1, dcfg.decimation)
        n_out = (cd.acq.n_samples + dec - 1) // dec
        rf = np.ascontiguousarray(rf, dtype=self._dt(prec))
        iq = np.zeros((cd.n_events, cd.probe.n_elements, n_out, 2), dtype=self._dt(prec))
        f = self._fn("orc_demodulate", prec)
        f.argtypes = [C.c_void_p, C.c_void_p, self._pt(prec), self._pt(prec)]
        f(C.byref(cd), C.byref(dcfg), _ptr(rf, self._pt(prec)), _ptr(iq, self._pt(prec)))
        return iq[..., 0] + 1j * iq[..., 1]

    def beamform(self, cd, data, points, n0, n1, bcfg, ev_begin=0, ev_end=-1, prec="f32"):
        dt = self._dt(prec)
        if cd.is_iq:
            d = np.ascontiguousarray(np.stack([np.real(data), np.imag(data)], -1), dtype=dt)
        else:
            d = np.ascontiguousarray(data, dtype=dt)
        pts = np.ascontiguousarray(points, dtype=np.float32)
        out = np.zeros((n0, n1, 2), dtype=dt)
        f = self._fn("orc_beamform", prec)
        f.argtypes = [C.c_void_p, self._pt(prec), C.c_int, C.c_int, f32p, C.c_void_p, C.c_int,
                      C.c_int, self._pt(prec)]
        f(C.byref(cd), _ptr(d, self._pt(prec)), n0, n1, _ptr(pts, f32p), C.byref(bcfg), ev_begin,
          ev_end, _ptr(out, self._pt(prec)))
        return out[..., 0] + 1j * out[..., 1]

    def mv_training_pairs(self, cd, data, points, n0, n1, bcfg, prec="f32"):
        """(frame, features [n_pix, 256], weights [n_pix, 128], valid [n_pix]) of
        the minimum-variance beamform (learned-MV training pairs)."""
        dt = self._dt(prec)
        d = np.ascontiguousarray(np.stack([np.real(data), np.imag(data)], -1), dtype=dt)
        pts = np.ascontiguousarray(points, dtype=np.float32)
        out = np.zeros((n0, n1, 2), dtype=dt)
        feat = np.zeros((n0 * n1, 256), dtype=dt)
        w = np.zeros((n0 * n1, 128), dtype=dt)
        valid = np.zeros(n0 * n1, dtype=np.uint8)
        f = self._fn("orc_mv_training_pairs", prec)
        f.argtypes = [C.c_void_p, self._pt(prec), C.c_int, C.c_int, f32p, C.c_void_p, self._pt(prec),
                      self._pt(prec), self._pt(prec), C.c_void_p]
        rc = f(C.byref(cd), _ptr(d, self._pt(prec)), n0, n1, _ptr(pts, f32p), C.byref(bcfg),
               _ptr(out, self._pt(prec)), _ptr(feat, self._pt(prec)), _ptr(w, self._pt(prec)), valid.ctypes.data)
        if rc != 0:
            raise ValueError("mv_training_pairs needs a coherent minimum-variance config")
        return out[..., 0] + 1j * out[..., 1], feat, w, valid

    def set_lmv_subspace(self, net_out128, n_beams: int, prec="f32"):
        """Make the MV combiner solve within span{n_beams + 1 DFT beams, the
        network output vector net_out128 / L} (None restores the exact solve)."""
        f = self._fn("orc_set_lmv_subspace", prec)
        f.argtypes = [f32p, C.c_int]
        f.restype = None
        if net_out128 is None:
            f(None, -1)
        else:
            v = np.ascontiguousarray(net_out128, dtype=np.float32)
            assert v.size == 128
            self._sub_keep = v
            f(_ptr(v, f32p), int(n_beams))

    def _cplx(self, a, prec):
        dt = self._dt(prec)
        return np.ascontiguousarray(np.stack([np.real(a), np.imag(a)], -1), dtype=dt)

    def wall_filter(self, ens, wtype, order, prec="f32"):
        e = self._cplx(ens, prec)
        out = np.zeros_like(e)
        n = ens.shape[0]
        n_pix = int(np.prod(ens.shape[1:]))
        f = self._fn("orc_wall_filter", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_long, C.c_int, C.c_int, self._pt(prec)]
        f(_ptr(e, self._pt(prec)), n, n_pix, wtype, order, _ptr(out, self._pt(prec)))
        return out[..., 0] + 1j * out[..., 1]

    def color_flow(self, ens, axis1, fdem, prf, c, dcfg, prec="f32"):
        e = self._cplx(ens, prec)
        n, n0, n1 = ens.shape
        dt = self._dt(prec)
        vel, pw, var = (np.zeros((n0, n1), dt) for _ in range(3))
        valid = np.zeros((n0, n1), np.uint8)
        nyq = (C.c_float if prec == "f32" else C.c_double)()
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        f = self._fn("orc_color_flow", prec)
        rt = C.c_float if prec == "f32" else C.c_double
        f.argtypes = [self._pt(prec), C.c_int, C.c_int, C.c_int, f32p, C.c_float, rt, rt,
                      C.c_void_p, self._pt(prec), self._pt(prec), self._pt(prec), u8p, C.c_void_p]
        f(_ptr(e, self._pt(prec)), n, n0, n1, _ptr(ax, f32p), fdem, prf, c, C.byref(dcfg),
          _ptr(vel, self._pt(prec)), _ptr(pw, self._pt(prec)), _ptr(var, self._pt(prec)),
          _ptr(valid, u8p), C.byref(nyq))
        return vel, pw, var, valid, nyq.value

    def power_doppler(self, ens, wtype, order, prec="f32"):
        e = self._cplx(ens, prec)
        n = ens.shape[0]
        n_pix = int(np.prod(ens.shape[1:]))
        out = np.zeros(ens.shape[1:], self._dt(prec))
        f = self._fn("orc_power_doppler", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_long, C.c_int, C.c_int, self._pt(prec)]
        f(_ptr(e, self._pt(prec)), n, n_pix, wtype, order, _ptr(out, self._pt(prec)))
        return out

    def displacement(self, a, b, axis1, fdem, c, ka=8, kl=2, max_lag=8, prec="f32"):
        n0, n1 = a.shape
        A, B = self._cplx(a, prec), self._cplx(b, prec)
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        axial = np.zeros((n0, n1), self._dt(prec))
        corr = np.zeros((n0, n1), self._dt(prec))
        rt = C.c_float if prec == "f32" else C.c_double
        f = self._fn("orc_axial_displacement", prec)
        f.argtypes = [self._pt(prec), self._pt(prec), C.c_int, C.c_int, f32p, C.c_float, rt,
                      C.c_int, C.c_int, C.c_int, self._pt(prec), self._pt(prec)]
        f(_ptr(A, self._pt(prec)), _ptr(B, self._pt(prec)), n0, n1, _ptr(ax, f32p), fdem, c, ka,
          kl, max_lag, _ptr(axial, self._pt(prec)), _ptr(corr, self._pt(prec)))
        return axial, corr

    def strain(self, axial, axis1, fit=15, prec="f32"):
        n0, n1 = axial.shape
        a = np.ascontiguousarray(axial, dtype=self._dt(prec))
        ax = np.ascontiguousarray(axis1, dtype=np.float32)
        out = np.zeros((n0, n1), self._dt(prec))
        f = self._fn("orc_axial_strain", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_int, f32p, C.c_int, self._pt(prec)]
        f(_ptr(a, self._pt(prec)), n0, n1, _ptr(ax, f32p), fit, _ptr(out, self._pt(prec)))
        return out

    def envelope(self, frame, fdem, prec="f32"):
        n0, n1 = frame.shape
        fr = self._cplx(frame, prec)
        out = np.zeros((n0, n1), self._dt(prec))
        f = self._fn("orc_envelope", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_int, C.c_float, self._pt(prec)]
        f(_ptr(fr, self._pt(prec)), n0, n1, fdem, _ptr(out, self._pt(prec)))
        return out

    def apply_tgc(self, env, points, atten, f0, prec="f32"):
        n0, n1 = env.shape
        e = np.ascontiguousarray(env, dtype=self._dt(prec))
        pts = np.ascontiguousarray(points, dtype=np.float32)
        out = np.zeros_like(e)
        rt = C.c_float if prec == "f32" else C.c_double
        f = self._fn("orc_apply_tgc", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_int, f32p, rt, rt, self._pt(prec)]
        f(_ptr(e, self._pt(prec)), n0, n1, _ptr(pts, f32p), atten, f0, _ptr(out, self._pt(prec)))
        return out

    def log_compress(self, env, dr=60.0, gain=0.0, ref=-1.0, prec="f32"):
        e = np.ascontiguousarray(env, dtype=self._dt(prec))
        out = np.zeros_like(e)
        rt = C.c_float if prec == "f32" else C.c_double
        f = self._fn("orc_log_compress", prec)
        f.argtypes = [self._pt(prec), C.c_long, rt, rt, rt, self._pt(prec)]
        f(_ptr(e, self._pt(prec)), e.size, dr, gain, ref, _ptr(out, self._pt(prec)))
        return out

    def scan_convert(self, img, grid_type, axis0, axis1, apex, points, width, height, fill=0.0,
                     prec="f32"):
        n0, n1 = img.shape
        im = np.ascontiguousarray(img, dtype=self._dt(prec))
        a0 = np.ascontiguousarray(axis0, dtype=np.float32)
        a1 = np.ascontiguousarray(axis1, dtype=np.float32)
        ap = np.ascontiguousarray(apex, dtype=np.float32)
        pts = np.ascontiguousarray(points, dtype=np.float32)
        px = np.zeros((height, width), self._dt(prec))
        ext = np.zeros(4, self._dt(prec))
        rt = C.c_float if prec == "f32" else C.c_double
        f = self._fn("orc_scan_convert", prec)
        f.argtypes = [self._pt(prec), C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_int,
                      C.c_int, rt, self._pt(prec), self._pt(prec)]
        f(_ptr(im, self._pt(prec)), grid_type, n0, n1, _ptr(a0, f32p), _ptr(a1, f32p),
          _ptr(ap, f32p), _ptr(pts, f32p), width, height, fill, _ptr(px, self._pt(prec)),
          _ptr(ext, self._pt(prec)))
        return px, ext

    def set_threads(self, n):
        self.lib.orc_set_num_threads(int(n))

    def num_threads(self):
        return int(self.lib.orc_num_threads())


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


class RefLib:
    """The reference engine itself (oracle/_ref/libusx_ref.so), through ref_shim.cpp.

    Only where the reference checkout was present at build time; used to pin the
    oracle and to generate golden fixtures."""

    def __init__(self):
        if not REF_SO.exists():
            raise FileNotFoundError(f"{REF_SO} not built")
        self.lib = C.CDLL(str(REF_SO))

    def speckle_box(self, x_min, x_max, z_min, z_max, y_half, n, seed=1234, sigma=1.0):
        out = np.zeros((n, 8), np.float32)
        f = self.lib.ref_speckle_box
        f.argtypes = [C.c_float] * 5 + [C.c_int, C.c_uint, C.c_float, f32p]
        f(x_min, x_max, z_min, z_max, y_half, n, seed, sigma, _ptr(out, f32p))
        return out

    def scale_in_circle(self, scat, cx, cz, radius, scale):
        s = np.ascontiguousarray(scat, dtype=np.float32).copy()
        f = self.lib.ref_scale_in_circle
        f.argtypes = [f32p, C.c_long, C.c_float, C.c_float, C.c_float, C.c_float]
        f(_ptr(s, f32p), len(s), cx, cz, radius, scale)
        return s

    def flow_tube(self, cx, cz, radius, length, angle, v_peak, n, seed=99, amplitude=0.05):
        out = np.zeros((n, 8), np.float32)
        f = self.lib.ref_flow_tube
        f.argtypes = [C.c_float] * 6 + [C.c_int, C.c_uint, C.c_float, f32p]
        f(cx, cz, radius, length, angle, v_peak, n, seed, amplitude, _ptr(out, f32p))
        return out

    def transmits(self, pr, med, kind, params, window=1, f_number=2.0):
        """kind: 'plane' (params = angles), 'focused' ((x, focal_depth, angle) tuples),
        'diverging' ((angle, vs_depth) tuples). Mirrors Simulator::make_* ."""
        n_el = pr.n_elements
        rows = []
        for p in params:
            t = Transmit()
            if kind == "plane":
                t.type, t.angle = 1, float(p)
            elif kind == "focused":
                x, fd, a = p
                t.type, t.angle = 0, float(a)
                t.origin[0] = float(x)
                t.focus[0] = float(np.float32(x) + np.float32(fd) * np.float32(np.tan(np.float32(a))))
                t.focus[2] = float(fd)
            else:
                a, vs = p
                t.type, t.angle = 2, float(a)
                t.focus[0] = float(-np.float32(vs) * np.float32(np.tan(np.float32(a))))
                t.focus[2] = float(-vs)
            d = np.zeros(n_el, np.float32)
            ap = np.zeros(n_el, np.float32)
            f = self.lib.ref_transmit_delays
            f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float, f32p, f32p]
            f.restype = C.c_float
            f(C.byref(pr), C.byref(med), C.byref(t), window, f_number, _ptr(d, f32p), _ptr(ap, f32p))
            rows.append((t.type, t.angle, tuple(t.focus), tuple(t.origin), d, ap))
        return TxSet(np.array([r[0] for r in rows], np.int32), np.array([r[1] for r in rows], np.float32),
                     np.array([r[2] for r in rows], np.float32), np.array([r[3] for r in rows], np.float32),
                     np.stack([r[4] for r in rows]), np.stack([r[5] for r in rows]))

    def grid(self, gtype, a0_min, a0_max, n0, a1_min, a1_max, n1, apex=(0.0, 0.0, 0.0)):
        ax0 = np.zeros(n0, np.float32)
        ax1 = np.zeros(n1, np.float32)
        pts = np.zeros((n0 * n1, 3), np.float32)
        ap = np.asarray(apex, np.float32)
        f = self.lib.ref_grid
        f.argtypes = [C.c_int, C.c_float, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, f32p,
                      f32p, f32p, f32p]
        f(gtype, a0_min, a0_max, n0, a1_min, a1_max, n1, _ptr(ap, f32p), _ptr(ax0, f32p),
          _ptr(ax1, f32p), _ptr(pts, f32p))
        return ax0, ax1, pts

    def normals(self, seed, n):
        out = np.zeros(n, np.float32)
        f = self.lib.ref_normals
        f.argtypes = [C.c_uint, C.c_long, f32p]
        f(seed, n, _ptr(out, f32p))
        return out

    def simulate(self, cd, scfg, scat):
        scat = np.ascontiguousarray(scat, dtype=np.float32)
        rf = np.zeros((cd.n_events, cd.probe.n_elements, cd.acq.n_samples), np.float32)
        f = self.lib.ref_simulate
        f.argtypes = [C.c_void_p, C.c_void_p, f32p, C.c_long, f32p]
        f(C.byref(cd), C.byref(scfg), _ptr(scat, f32p), len(scat), _ptr(rf, f32p))
        return rf

    def pulse(self, cd, scfg):
        f = self.lib.ref_pulse
        f.argtypes = [C.c_void_p, C.c_void_p, f32p, f32p]
        n = f(C.byref(cd), C.byref(scfg), None, None)
        p = np.zeros(n, np.float32)
        h = C.c_float()
        f(C.byref(cd), C.byref(scfg), _ptr(p, f32p), C.byref(h))
        return p, h.value

    def demodulate(self, cd, dcfg, rf):
        dec = max(1, dcfg.decimation)
        n_out = (cd.acq.n_samples + dec - 1) // dec
        rf = np.ascontiguousarray(rf, dtype=np.float32)
        iq = np.zeros((cd.n_events, cd.probe.n_elements, n_out), np.complex64)
        f = self.lib.ref_demodulate
        f.argtypes = [C.c_void_p, C.c_void_p, f32p, C.c_void_p]
        f(C.byref(cd), C.byref(dcfg), _ptr(rf, f32p), iq.ctypes.data)
        return iq

    def beamform(self, cd, data, gtype, axis0, axis1, apex, points, bcfg, ev_begin=0, ev_end=-1):
        n0, n1 = len(axis0), len(axis1)
        d = np.ascontiguousarray(data, dtype=np.complex64 if cd.is_iq else np.float32)
        out = np.zeros((n0, n1), np.complex64)
        a0 = np.ascontiguousarray(axis0, np.float32)
        a1 = np.ascontiguousarray(axis1, np.float32)
        ap = np.ascontiguousarray(apex, np.float32)
        pts = np.ascontiguousarray(points, np.float32)
        f = self.lib.ref_beamform
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, f32p,
                      C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        f(C.byref(cd), d.ctypes.data, gtype, n0, n1, _ptr(a0, f32p), _ptr(a1, f32p), _ptr(ap, f32p),
          _ptr(pts, f32p), C.byref(bcfg), ev_begin, ev_end, out.ctypes.data)
        return out

    def wall_filter(self, ens, axis1, wtype, order):
        e = np.ascontiguousarray(ens, np.complex64)
        n, n0, n1 = e.shape
        out = np.zeros_like(e)
        ax = np.ascontiguousarray(axis1, np.float32)
        f = self.lib.ref_wall_filter
        f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, C.c_int, C.c_int, C.c_void_p]
        f(e.ctypes.data, n, n0, n1, _ptr(ax, f32p), wtype, order, out.ctypes.data)
        return out

    def color_flow(self, ens, axis1, fdem, prf, c, dcfg):
        e = np.ascontiguousarray(ens, np.complex64)
        n, n0, n1 = e.shape
        vel, pw, var = (np.zeros((n0, n1), np.float32) for _ in range(3))
        valid = np.zeros((n0, n1), np.uint8)
        ax = np.ascontiguousarray(axis1, np.float32)
        f = self.lib.ref_color_flow
        f.restype = C.c_float
        f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_float,
                      C.c_void_p, f32p, f32p, f32p, u8p]
        nyq = f(e.ctypes.data, n, n0, n1, _ptr(ax, f32p), fdem, prf, c, C.byref(dcfg),
                _ptr(vel, f32p), _ptr(pw, f32p), _ptr(var, f32p), _ptr(valid, u8p))
        return vel, pw, var, valid, nyq

    def power_doppler(self, ens, axis1, wtype, order):
        e = np.ascontiguousarray(ens, np.complex64)
        n, n0, n1 = e.shape
        out = np.zeros((n0, n1), np.float32)
        ax = np.ascontiguousarray(axis1, np.float32)
        f = self.lib.ref_power_doppler
        f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, C.c_int, C.c_int, f32p]
        f(e.ctypes.data, n, n0, n1, _ptr(ax, f32p), wtype, order, _ptr(out, f32p))
        return out

    def displacement(self, a, b, axis1, fdem, c, ka=8, kl=2, max_lag=8):
        A = np.ascontiguousarray(a, np.complex64)
        B = np.ascontiguousarray(b, np.complex64)
        n0, n1 = A.shape
        axial = np.zeros((n0, n1), np.float32)
        corr = np.zeros((n0, n1), np.float32)
        ax = np.ascontiguousarray(axis1, np.float32)
        f = self.lib.ref_displacement
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int,
                      C.c_int, C.c_int, f32p, f32p]
        f(A.ctypes.data, B.ctypes.data, n0, n1, _ptr(ax, f32p), fdem, c, ka, kl, max_lag,
          _ptr(axial, f32p), _ptr(corr, f32p))
        return axial, corr

    def strain(self, axial, axis1, fit=15):
        a = np.ascontiguousarray(axial, np.float32)
        n0, n1 = a.shape
        out = np.zeros((n0, n1), np.float32)
        ax = np.ascontiguousarray(axis1, np.float32)
        f = self.lib.ref_strain
        f.argtypes = [f32p, C.c_int, C.c_int, f32p, C.c_int, f32p]
        f(_ptr(a, f32p), n0, n1, _ptr(ax, f32p), fit, _ptr(out, f32p))
        return out

    def envelope(self, frame, gtype, axis0, axis1, apex, points, fdem):
        fr = np.ascontiguousarray(frame, np.complex64)
        n0, n1 = fr.shape
        out = np.zeros((n0, n1), np.float32)
        args = [np.ascontiguousarray(x, np.float32) for x in (axis0, axis1, apex, points)]
        f = self.lib.ref_envelope
        f.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_float, f32p]
        f(fr.ctypes.data, gtype, n0, n1, *[_ptr(x, f32p) for x in args], fdem, _ptr(out, f32p))
        return out

    def apply_tgc(self, env, gtype, axis0, axis1, apex, points, atten, f0):
        e = np.ascontiguousarray(env, np.float32)
        n0, n1 = e.shape
        out = np.zeros_like(e)
        args = [np.ascontiguousarray(x, np.float32) for x in (axis0, axis1, apex, points)]
        f = self.lib.ref_apply_tgc
        f.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_float,
                      C.c_float, f32p]
        f(_ptr(e, f32p), gtype, n0, n1, *[_ptr(x, f32p) for x in args], atten, f0, _ptr(out, f32p))
        return out

    def log_compress(self, env, dr=60.0, gain=0.0, ref=-1.0):
        e = np.ascontiguousarray(env, np.float32)
        out = np.zeros_like(e)
        f = self.lib.ref_log_compress
        f.argtypes = [f32p, C.c_long, C.c_float, C.c_float, C.c_float, f32p]
        f(_ptr(e, f32p), e.size, dr, gain, ref, _ptr(out, f32p))
        return out

    def scan_convert(self, img, gtype, axis0, axis1, apex, points, width, height, fill=0.0):
        im = np.ascontiguousarray(img, np.float32)
        n0, n1 = im.shape
        px = np.zeros((height, width), np.float32)
        ext = np.zeros(4, np.float32)
        args = [np.ascontiguousarray(x, np.float32) for x in (axis0, axis1, apex, points)]
        f = self.lib.ref_scan_convert
        f.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_int, C.c_int,
                      C.c_float, f32p, f32p]
        f(_ptr(im, f32p), gtype, n0, n1, *[_ptr(x, f32p) for x in args], width, height, fill,
          _ptr(px, f32p), _ptr(ext, f32p))
        return px, ext
