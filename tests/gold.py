"""Helpers that rebuild C descriptors from the golden fixtures (shared by the
oracle tests and the GPU parity tests)."""

from __future__ import annotations

import numpy as np

from oracle import oracle as O


def sim_setup(g):
    p = g["probe"]
    a = g["acq"]
    pr = O.probe(n_elements=int(p[0]), pitch=float(p[1]), element_width=float(p[2]),
                 center_frequency=float(p[3]), bandwidth=float(p[4]))
    acq = O.acquisition(fs=float(a[0]), n_samples=int(a[1]), t0=float(a[2]), prf=float(a[3]))
    return pr, O.medium(), acq


def txset(g, prefix):
    return O.TxSet(g[f"{prefix}_types"], g[f"{prefix}_angles"], g[f"{prefix}_focus"], g[f"{prefix}_origin"],
                   g[f"{prefix}_delays"], g[f"{prefix}_apod"])


BF_CASES = {
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


def rel_l2(a, b) -> float:
    a = np.asarray(a).astype(np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b).astype(a.dtype)
    d = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (d if d > 0 else 1.0))
