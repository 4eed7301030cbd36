"""Image-quality metrics: contrast, CNR, rank-binned gCNR, speckle SNR and
point-spread-function width. Same definitions, masks and binning as the
reference's python/usx/metrics.py, so numbers are comparable one to one."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

RAYLEIGH_SPECKLE_SNR = 1.9137


def _regions(grid, center_xz, radius, background=(1.6, 2.6), inner_scale=0.7):
    x = np.asarray(grid.axis0)[:, None]
    z = np.asarray(grid.axis1)[None, :]
    r = np.hypot(x - center_xz[0], z - center_xz[1])
    inside = r <= radius * inner_scale
    outside = (r > radius * background[0]) & (r < radius * background[1])
    return inside, outside, r


def contrast_db(env, grid, center_xz, radius, background=(1.6, 2.6)) -> float:
    """Mean-power ratio of lesion (0.7 r) to background annulus, in dB."""
    inside, outside, _ = _regions(grid, center_xz, radius, background)
    e = np.asarray(env, dtype=np.float64)
    p_in = np.mean(e[inside] ** 2)
    p_out = np.mean(e[outside] ** 2)
    return float(10.0 * np.log10((p_in + 1e-30) / (p_out + 1e-30)))


def cnr(env, grid, center_xz, radius, background=(1.6, 2.6)) -> float:
    """|mu_in - mu_out| / sqrt(var_in + var_out)."""
    inside, outside, _ = _regions(grid, center_xz, radius, background)
    e = np.asarray(env, dtype=np.float64)
    a, b = e[inside], e[outside]
    return float(abs(a.mean() - b.mean()) / (np.sqrt(a.var() + b.var()) + 1e-30))


def gcnr(env, grid, center_xz, radius, background=(1.6, 2.6), bins: int = 100) -> float:
    """Generalized CNR, 1 - overlap of the two regions' distributions, with the
    histograms taken over pooled ranks so the value is invariant under any
    monotone transform of the pixel values."""
    inside, outside, _ = _regions(grid, center_xz, radius, background)
    e = np.asarray(env, dtype=np.float64)
    a, b = e[inside], e[outside]
    if a.size == 0 or b.size == 0:
        return 0.0
    pooled = np.sort(np.concatenate([a, b]))
    scale = max(pooled.size - 1, 1)
    ra = np.searchsorted(pooled, a, side="left") / scale
    rb = np.searchsorted(pooled, b, side="left") / scale
    edges = np.linspace(0.0, 1.0, bins + 1)
    ha = np.histogram(ra, bins=edges)[0]
    hb = np.histogram(rb, bins=edges)[0]
    ha = ha / max(ha.sum(), 1)
    hb = hb / max(hb.sum(), 1)
    return float(1.0 - np.minimum(ha, hb).sum())


def speckle_snr(env, grid, region_xz, half_size, detrend: bool = True) -> float:
    """mu / sigma of the envelope in a rectangle, optionally after dividing out
    the mean along each axis (attenuation and aperture gain profiles)."""
    x = np.asarray(grid.axis0)
    z = np.asarray(grid.axis1)
    mx = np.abs(x - region_xz[0]) <= half_size[0]
    mz = np.abs(z - region_xz[1]) <= half_size[1]
    v = np.asarray(env, dtype=np.float64)[np.ix_(mx, mz)]
    if v.size == 0:
        return float("nan")
    if detrend and v.shape[0] > 1 and v.shape[1] > 1:
        v = v / np.maximum(v.mean(axis=0, keepdims=True), 1e-30)
        v = v / np.maximum(v.mean(axis=1, keepdims=True), 1e-30)
    return float(v.mean() / (v.std() + 1e-30))


@dataclass
class PointSpreadFunction:
    x: float
    z: float
    lateral_fwhm: float
    axial_fwhm: float
    peak: float
    sidelobe_db: float

    def __repr__(self) -> str:
        return (f"PSF(x={self.x*1e3:.2f}mm z={self.z*1e3:.2f}mm lateral={self.lateral_fwhm*1e3:.3f}mm "
                f"axial={self.axial_fwhm*1e3:.3f}mm sidelobe={self.sidelobe_db:.1f}dB)")


def _fwhm(axis, profile) -> float:
    """Full width at half maximum, half-power crossings linearly interpolated."""
    p = np.asarray(profile, dtype=np.float64)
    i = int(np.argmax(p))
    half = 0.5 * p[i]
    if p[i] <= 0:
        return float("nan")

    def edge(step):
        j = i
        while 0 <= j + step < len(p) and p[j + step] > half:
            j += step
        k = j + step
        if not 0 <= k < len(p):
            return float(axis[j])
        t = (half - p[j]) / (p[k] - p[j])
        return float(axis[j] + t * (axis[k] - axis[j]))

    return abs(edge(1) - edge(-1))


def measure_psf(env, grid, near_xz, search_radius: float = 0.002) -> PointSpreadFunction:
    """PSF of the brightest target within `search_radius` of `near_xz`."""
    e = np.asarray(env, dtype=np.float64)
    ax0 = np.asarray(grid.axis0)
    ax1 = np.asarray(grid.axis1)
    r = np.hypot(ax0[:, None] - near_xz[0], ax1[None, :] - near_xz[1])
    win = r <= search_radius
    if not win.any():
        raise ValueError("no pixels within the search radius")
    i, j = np.unravel_index(np.argmax(np.where(win, e, -np.inf)), e.shape)
    lat = _fwhm(ax0, e[:, j])
    axi = _fwhm(ax1, e[i, :])
    dist = np.hypot(ax0[:, None] - ax0[i], ax1[None, :] - ax1[j])
    region = (dist > max(3 * lat, 3 * axi, 5e-4)) & win
    peak = e[i, j]
    side = (float(20 * np.log10((e[region].max() + 1e-30) / (peak + 1e-30))) if region.any() else float("nan"))
    return PointSpreadFunction(x=float(ax0[i]), z=float(ax1[j]), lateral_fwhm=lat, axial_fwhm=axi,
                               peak=float(peak), sidelobe_db=side)


def summarize(env, grid, lesion_xz=None, lesion_radius=None, wire_xz=None, speckle_xz=None,
              speckle_half=(0.004, 0.004)) -> dict:
    """All metrics that the arguments allow, as a plain dict."""
    out = {}
    if lesion_xz is not None and lesion_radius:
        out["contrast_db"] = contrast_db(env, grid, lesion_xz, lesion_radius)
        out["cnr"] = cnr(env, grid, lesion_xz, lesion_radius)
        out["gcnr"] = gcnr(env, grid, lesion_xz, lesion_radius)
    if wire_xz is not None:
        psf = measure_psf(env, grid, wire_xz)
        out["lateral_fwhm_mm"] = psf.lateral_fwhm * 1e3
        out["axial_fwhm_mm"] = psf.axial_fwhm * 1e3
        out["sidelobe_db"] = psf.sidelobe_db
    if speckle_xz is not None:
        out["speckle_snr"] = speckle_snr(env, grid, speckle_xz, speckle_half)
    return out
