"""Learned minimum variance: training pairs, on-device training, evaluation.

The surrogate is a 4-layer fully connected network (256 -> 256 -> 256 -> 256
-> 128, ReLU, BF16 weights and activations with FP32 accumulation) that maps a
pixel's 256 minimum-variance features (normalised diagonal sums of the
spatially smoothed covariance and the subarray-averaged snapshot, computed by
the library's feature kernel) to its Capon weights L w / sum(w). Training
pairs come from the plain tensor-core minimum variance run on simulated
phantoms (the plan's training export); training runs on the device through
usx_cu_mlp_train_step (hand-written forward/backward GEMMs and Adam). At
inference the plan gates each pixel on |1^H w - 1| and solves the rejected
ones exactly, so plain minimum variance is both the fallback and the
reference the image metrics are compared against.

    python -m usx.learned train --phantoms 200 --out weights.bin
    python -m usx.learned evaluate --weights weights.bin --phantoms 16

No counterpart in the reference; its minimum variance is
core/src/beamformer.cpp:137-214.
"""

from __future__ import annotations

import argparse
import json
import math
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import capi

DIMS = (256, 256, 256, 256, 128)
FEATURES, OUTPUTS = DIMS[0], DIMS[-1]
DEFAULT_GATE = 0.05
# Subspace refinement: the exact Capon solve within span{network weights,
# look direction, DFT beams +-1, +-2} (usx_cu_bf_plan_set_learned_refine).
DEFAULT_REFINE = 4
COMB_MV, COMB_LEARNED_MV = 2, 3
MAGIC = b"USXMLP1\0"
DEFAULT_WEIGHTS = Path(__file__).resolve().parents[2] / "weights" / "learned_mv_128ch_l64.bin"


# ------------------------------------------------------------------ weights file

def save_weights(path, dims, params) -> None:
    """Raw little-endian file: magic, int32 n_layers, int32 dims[n+1], float32 params."""
    dims = np.asarray(dims, np.int32)
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.int32(len(dims) - 1).tobytes())
        f.write(dims.astype("<i4").tobytes())
        f.write(np.ascontiguousarray(params, dtype="<f4").tobytes())


def load_weights(path):
    """(dims, params) from a file written by save_weights."""
    raw = Path(path).read_bytes()
    if raw[:8] != MAGIC:
        raise ValueError(f"{path}: not a usx network file")
    n = int(np.frombuffer(raw, "<i4", 1, 8)[0])
    dims = tuple(int(d) for d in np.frombuffer(raw, "<i4", n + 1, 12))
    params = np.frombuffer(raw, "<f4", offset=12 + 4 * (n + 1)).copy()
    expect = sum(a * b + b for a, b in zip(dims[:-1], dims[1:]))
    if params.size != expect:
        raise ValueError(f"{path}: {params.size} parameters, expected {expect}")
    return dims, params


# ------------------------------------------------------------------ geometry

@dataclass
class Setup:
    """Probe, acquisition and grid of the 128-channel 75-plane-wave 512 x 1024
    configuration (the shapes the surrogate is trained for)."""
    n_el: int = 128
    pitch: float = 300e-6
    width: float = 270e-6
    f0: float = 5e6
    fs: float = 20e6
    c: float = 1540.0
    n_tx: int = 75
    max_angle_deg: float = 16.0
    depth: float = 0.060
    z0: float = 0.005
    n0: int = 512
    n1: int = 1024
    f_number: float = 1.5
    subarray: int = 64
    loading: float = 0.01
    range_avg: int = 2

    def build(self):
        """(ch_rf, ch_iq, grid, n_samples, transmits) capi descriptors; transmit
        delays from the host library."""
        import usx
        probe = usx.Probe()
        probe.n_elements, probe.pitch, probe.element_width = self.n_el, self.pitch, self.width
        probe.center_frequency, probe.bandwidth = self.f0, 0.6
        medium = usx.Medium()
        acq = usx.presets.acquisition(probe, depth=self.depth, medium=medium, samples_per_wavelength=self.fs / self.f0)
        sim = usx.Simulator(probe, medium, acq, usx.SimulatorConfig())
        txs = sim.make_plane_waves(usx.angles_deg(-self.max_angle_deg, self.max_angle_deg, self.n_tx))
        tx = [dict(type=1, angle=t.angle, delays=t.delays, apodization=t.apodization) for t in txs]
        cp = capi.Probe(self.n_el, probe.pitch, probe.element_width, probe.elevation_height, self.f0, probe.bandwidth)
        cm = capi.Medium(medium.speed_of_sound, medium.attenuation, medium.density)
        ca = capi.Acquisition(acq.sampling_frequency, acq.n_samples, acq.t0, acq.prf)
        ch_rf = capi.Channel(cp, cm, ca, tx)
        ch_iq = capi.Channel(cp, cm, ca, tx, is_iq=True, fdem=self.f0)
        grid = usx.grid_for(probe, self.z0, self.depth, self.n0, self.n1)
        cgrid = capi.Grid(0, np.asarray(grid.axis0), np.asarray(grid.axis1), np.asarray(grid.points).reshape(-1, 3))
        return ch_rf, ch_iq, cgrid, acq.n_samples, tx

    def bf(self, combiner: int) -> capi.BeamformerConfig:
        return capi.bf_config(f_number=self.f_number, combiner=combiner, mv_subarray=self.subarray,
                              mv_diagonal_loading=self.loading, mv_range_average=self.range_avg)

    @property
    def half_width(self) -> float:
        return 0.5 * (self.n_el - 1) * self.pitch


# ------------------------------------------------------------------ phantoms

@dataclass
class PhantomSpec:
    scatterers: np.ndarray      # [n, 8] float32 (x, y, z, amplitude, vx, vy, vz, pad)
    cysts: list                 # [(x, z, r)]
    wires: list                 # [(x, z, amplitude)]


def phantom(seed: int, setup: Setup = Setup()) -> PhantomSpec:
    """Seeded speckle phantom: 50k-150k N(0,1) scatterers over the imaged
    region, 1-3 anechoic cysts of radius 1-5 mm and 2-6 wires of amplitude
    5-50 (numpy PCG64 stream `seed`). Cysts and wires keep 3 mm apart."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(50_000, 150_001))
    xh = 1.1 * setup.half_width
    pos = np.stack([rng.uniform(-xh, xh, n), np.zeros(n), rng.uniform(setup.z0 - 1e-3, setup.depth + 2e-3, n)], 1)
    amp = rng.standard_normal(n)
    cysts, wires = [], []
    for _ in range(int(rng.integers(1, 4))):
        for _try in range(50):
            r = rng.uniform(1e-3, 5e-3)
            x, z = rng.uniform(-0.8 * xh, 0.8 * xh), rng.uniform(setup.z0 + 2 * r + 2e-3, setup.depth - 2 * r - 2e-3)
            if all(math.hypot(x - cx, z - cz) > r + cr + 3e-3 for cx, cz, cr in cysts):
                cysts.append((x, z, r))
                break
    keep = np.ones(n, bool)
    for x, z, r in cysts:
        keep &= np.hypot(pos[:, 0] - x, pos[:, 2] - z) > r
    pos, amp = pos[keep], amp[keep]
    for _ in range(int(rng.integers(2, 7))):
        for _try in range(50):
            x, z = rng.uniform(-0.85 * setup.half_width, 0.85 * setup.half_width), rng.uniform(setup.z0 + 3e-3,
                                                                                                setup.depth - 3e-3)
            if all(math.hypot(x - cx, z - cz) > cr + 3e-3 for cx, cz, cr in cysts) and \
                    all(math.hypot(x - wx, z - wz) > 3e-3 for wx, wz, _ in wires):
                wires.append((x, z, float(rng.uniform(5.0, 50.0))))
                break
    if wires:
        pos = np.concatenate([pos, np.array([[x, 0.0, z] for x, z, _ in wires])])
        amp = np.concatenate([amp, np.array([a for _, _, a in wires])])
    s = np.zeros((len(amp), 8), np.float32)
    s[:, 0:3] = pos
    s[:, 3] = amp
    return PhantomSpec(s, cysts, wires)


# ------------------------------------------------------------------ acquisition

class Imager:
    """GPU simulation, demodulation and beamforming of phantoms in one context
    (the legacy default stream, so torch and the library share ordering)."""

    def __init__(self, setup: Setup = Setup(), device: int = 0, noise_db: float = -60.0):
        import torch
        self.torch = torch
        self.setup = setup
        self.ctx = capi.Context(device, stream=0)
        self.ch_rf, self.ch_iq, self.grid, self.n_smp, self.transmits = setup.build()
        self.sim_cfg = capi.sim_config(noise_db=noise_db)
        self.n_pix = setup.n0 * setup.n1
        self.rf = torch.empty((setup.n_tx, setup.n_el, self.n_smp), dtype=torch.float32, device="cuda")
        self.iq = torch.empty((setup.n_tx, setup.n_el, self.n_smp), dtype=torch.complex64, device="cuda")
        self.plans = {}

    def plan(self, combiner: int) -> capi.Plan:
        if combiner not in self.plans:
            p = self.ctx.plan(self.ch_iq, self.grid, self.setup.bf(combiner))
            if combiner == COMB_MV:
                p.set_mv_mode(1)
            self.plans[combiner] = p
        return self.plans[combiner]

    def acquire(self, spec: PhantomSpec, noise_seed: int = 0):
        """Simulate (with receive noise from seeded device normals) and demodulate into self.iq."""
        torch = self.torch
        scat = torch.from_numpy(spec.scatterers).cuda()
        gen = torch.Generator(device="cuda")
        gen.manual_seed(int(noise_seed) + 77)
        z = torch.randn(self.rf.shape, generator=gen, device="cuda", dtype=torch.float32)
        self.ctx.simulate(self.ch_rf, self.sim_cfg, scat.data_ptr(), scat.shape[0], z.data_ptr(),
                          self.rf.data_ptr())
        self.ctx.demodulate(self.ch_rf, capi.demod_config(), self.rf.data_ptr(), self.iq.data_ptr())
        self.ctx.synchronize()
        del scat, z

    def beamform(self, combiner: int):
        frame = self.torch.empty((self.setup.n0, self.setup.n1), dtype=self.torch.complex64, device="cuda")
        self.plan(combiner).execute(self.iq.data_ptr(), frame.data_ptr())
        return frame

    def export_pairs(self):
        """Plain tensor-core MV frame with every pixel's (features, weights, valid)."""
        torch = self.torch
        feat = torch.empty((self.n_pix, FEATURES), dtype=torch.float32, device="cuda")
        w = torch.empty((self.n_pix, OUTPUTS), dtype=torch.float32, device="cuda")
        valid = torch.empty(self.n_pix, dtype=torch.uint8, device="cuda")
        p = self.plan(COMB_MV)
        p.set_training_export(feat.data_ptr(), w.data_ptr(), valid.data_ptr())
        try:
            frame = self.beamform(COMB_MV)
        finally:
            p.set_training_export(None, None, None)
        return frame, feat, w, valid

    def close(self):
        for p in self.plans.values():
            p.close()
        self.plans = {}
        self.ctx.close()


def output_mask(feat):
    """1 for the outputs of weights i < L (L = 64 f[0]), 0 beyond."""
    torch = __import__("torch")
    L = torch.round(feat[:, 0] * 64.0)
    k = torch.arange(OUTPUTS, device=feat.device)
    return ((k[None, :] // 2) < L[:, None]).float()


def sample_rows(frame, valid, n: int, gen, points=None, spec: PhantomSpec | None = None):
    """n valid pixel rows: 50% uniform, 20% within 1.5 mm of a wire, 20% inside
    or within 1 mm of a cyst, 10% from the 2% brightest pixels. Point targets,
    their side lobes and the cyst interiors are where the Capon weights move
    the image metrics; uniform rows cover the speckle."""
    torch = __import__("torch")
    dev = frame.device
    ok = valid.bool()
    pools = [(torch.nonzero(ok, as_tuple=False).squeeze(1), 0.5)]
    if spec is not None and points is not None:
        pts = torch.as_tensor(points, device=dev).reshape(-1, 3)
        near_w = torch.zeros_like(ok)
        for x, z, _ in spec.wires:
            near_w |= torch.hypot(pts[:, 0] - x, pts[:, 2] - z) < 1.5e-3
        near_c = torch.zeros_like(ok)
        for x, z, r in spec.cysts:
            near_c |= torch.hypot(pts[:, 0] - x, pts[:, 2] - z) < r + 1e-3
        pools += [(torch.nonzero(ok & near_w, as_tuple=False).squeeze(1), 0.2),
                  (torch.nonzero(ok & near_c, as_tuple=False).squeeze(1), 0.2)]
    idx = pools[0][0]
    mag = frame.reshape(-1).abs()[idx]
    k = max(1, int(0.02 * idx.numel()))
    pools.append((idx[torch.topk(mag, k).indices], 0.1))
    total = sum(f for p, f in pools if p.numel())
    out = []
    for p, f in pools:
        if p.numel() == 0:
            continue
        m = int(round(n * f / total))
        out.append(p[torch.randint(p.numel(), (m,), generator=gen, device=dev)])
    rows = torch.cat(out)
    if rows.numel() < n:
        rows = torch.cat([rows, pools[0][0][torch.randint(pools[0][0].numel(), (n - rows.numel(),), generator=gen,
                                                          device=dev)]])
    return rows[:n]


def make_pairs(imager: Imager, seeds, per_phantom: int = 16384, log=print):
    """Training pairs from the plain MV on the phantoms `seeds` (device tensors)."""
    torch = imager.torch
    gen = torch.Generator(device="cuda")
    gen.manual_seed(12345)
    X, T = [], []
    t0 = time.time()
    for i, s in enumerate(seeds):
        spec = phantom(int(s), imager.setup)
        imager.acquire(spec, noise_seed=int(s))
        frame, feat, w, valid = imager.export_pairs()
        rows = sample_rows(frame, valid, per_phantom, gen, imager.grid.points, spec)
        X.append(feat[rows].clone())
        T.append(w[rows].clone())
        del feat, w, valid, frame
        if log and (i + 1) % 20 == 0:
            log(f"pairs: {i + 1}/{len(seeds)} phantoms, {time.time() - t0:.1f} s")
    X = torch.cat(X)
    T = torch.cat(T)
    return X, T, output_mask(X)


def train(ctx: capi.Context, X, T, M, steps: int = 6000, batch: int = 4096, lr: float = 1e-3, seed: int = 0,
          log=print, log_every: int = 500, loss: str = "output", beta: float = 0.02) -> tuple[capi.Mlp, list]:
    """Adam on minibatches drawn on the device, cosine learning-rate decay.
    loss="output": the combiner-output error against plain MV's (plus beta x
    the weight MSE); loss="mse": the weight MSE alone; loss="subspace": the
    direction of the Capon weights outside the refinement's DFT beams (plus
    beta x the weight MSE)."""
    torch = __import__("torch")
    mlp = capi.Mlp(ctx, DIMS, seed)
    kinds = {"output": capi.Mlp.LOSS_LMV_OUTPUT, "mse": capi.Mlp.LOSS_MSE, "subspace": capi.Mlp.LOSS_LMV_SUBSPACE}
    mlp.set_loss(kinds[loss], beta)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed + 1)
    n = X.shape[0]
    losses = []
    for step in range(steps):
        idx = torch.randint(n, (batch,), generator=gen, device=X.device)
        xb, tb, mb = X[idx].contiguous(), T[idx].contiguous(), M[idx].contiguous()
        lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        want = step % log_every == 0 or step == steps - 1
        loss, _ = mlp.train_step(xb.data_ptr(), tb.data_ptr(), mb.data_ptr(), batch, lr_t, want_loss=want)
        if want:
            losses.append((step, loss))
            if log:
                log(f"step {step}: loss {loss:.5f} lr {lr_t:.2e}")
    return mlp, losses


def validation_loss(mlp: capi.Mlp, X, T, M) -> float:
    """Masked mean squared error of the network on (X, T)."""
    torch = __import__("torch")
    n = X.shape[0] // 128 * 128
    Y = torch.empty((n, OUTPUTS), dtype=torch.float32, device=X.device)
    mlp.forward(X[:n].contiguous().data_ptr(), n, Y.data_ptr())
    torch.cuda.synchronize()
    d = (Y - T[:n]) * M[:n]
    return float((d * d).sum() / (n * OUTPUTS))


def image_metrics(frame, imager: Imager, spec: PhantomSpec) -> dict:
    """gCNR/CNR per cyst and lateral/axial FWHM per wire (envelope of the frame)."""
    from . import metrics
    env = frame.abs().cpu().numpy()
    g = imager.grid
    out = {"gcnr": [], "cnr": [], "lateral_fwhm_mm": [], "axial_fwhm_mm": []}
    for x, z, r in spec.cysts:
        out["gcnr"].append(metrics.gcnr(env, g, (x, z), r))
        out["cnr"].append(metrics.cnr(env, g, (x, z), r))
    for x, z, _ in spec.wires:
        psf = metrics.measure_psf(env, g, (x, z), 1e-3)
        out["lateral_fwhm_mm"].append(psf.lateral_fwhm * 1e3)
        out["axial_fwhm_mm"].append(psf.axial_fwhm * 1e3)
    return out


@dataclass(frozen=True)
class Mode:
    """One learned-MV setting evaluated against plain minimum variance: the gate
    on the network's distortionless residual, the gate on the share of the
    refinement's power reduction carried by the network's direction, and
    whether that direction is in the refinement's basis at all (False: the
    DFT beams alone, the ablation of the network)."""
    gate: float = math.inf
    share: float = math.inf
    use_net: bool = True
    level: float = math.inf
    window: tuple = (0, 0)   # the level gate's neighbourhood: +/- lateral lines, +/- depths

    @property
    def label(self) -> str:
        if not self.use_net:
            return "beams_only"
        base = f"gate={self.gate:g},share={self.share:g}"
        if math.isinf(self.level):
            return base
        base = f"{base},level={self.level:g}"
        return base if tuple(self.window) == (0, 0) else f"{base},win={self.window[0]}x{self.window[1]}"


def modes_for(gates=(), shares=(), ablation: bool = True, levels=(), level_shares=(math.inf,),
              windows=((0, 0),)) -> list:
    """Modes of each single gate, and of every level gate combined with each of
    `level_shares` (share gates) and each of `windows` (the level gate's
    neighbourhood)."""
    out = [Mode(gate=float(g)) for g in gates] + [Mode(share=float(x)) for x in shares]
    out += [Mode(share=float(x), level=float(v), window=tuple(w))
            for v in levels for x in level_shares for w in windows]
    if ablation:
        out.append(Mode(use_net=False))
    seen, uniq = set(), []
    for m in out:
        if m.label not in seen:
            seen.add(m.label)
            uniq.append(m)
    return uniq


def evaluate(imager: Imager, mlp: capi.Mlp, seeds, modes=(Mode(),), log=print,
             refine: int = DEFAULT_REFINE) -> dict:
    """Image metrics of plain MV and of the learned MV in each mode on the
    held-out phantoms `seeds`: {mode label: summary}."""
    learned = imager.plan(COMB_LEARNED_MV)
    learned.set_learned_refine(refine)
    rows = {m.label: [] for m in modes}
    for s in seeds:
        spec = phantom(int(s), imager.setup)
        imager.acquire(spec, noise_seed=int(s))
        ref = imager.beamform(COMB_MV)
        a = image_metrics(ref, imager, spec)
        for m in modes:
            learned.set_learned(mlp, m.gate)
            learned.set_learned_subspace(m.use_net, m.share)
            learned.set_learned_level_gate(m.level)
            learned.set_learned_level_window(*m.window)
            learned.learned_stats()
            lf = imager.beamform(COMB_LEARNED_MV)
            gated, pixels = learned.learned_stats()
            b = image_metrics(lf, imager, spec)
            d = {k: [y - x for x, y in zip(a[k], b[k])] for k in a}
            rows[m.label].append({"seed": int(s), "plain": a, "learned": b, "delta": d,
                                  "fallback_rate": gated / max(1, pixels),
                                  "rel_l2": float((lf - ref).abs().pow(2).sum().sqrt()
                                                  / ref.abs().pow(2).sum().sqrt())})
        learned.set_learned_subspace(True, math.inf)
        learned.set_learned_level_gate(math.inf)
        learned.set_learned_level_window(0, 0)
        if log:
            log(f"phantom {s}: " + ", ".join(
                f"{m.label}: fallback {rows[m.label][-1]['fallback_rate']:.3f} dgcnr "
                f"{max([abs(v) for v in rows[m.label][-1]['delta']['gcnr']] or [0]):.4f}" for m in modes))
    return {label: summarize(r) for label, r in rows.items()}


def meets_bar(r: dict, max_dgcnr: float = 0.01, max_fwhm: float = 0.01) -> bool:
    """Held-out summary within the quality bar: every cyst's |delta gCNR| <=
    max_dgcnr and every wire's lateral and axial FWHM within max_fwhm
    (relative) of plain minimum variance."""
    if r.get("gcnr", {}).get("max_abs_delta", 1.0) > max_dgcnr:
        return False
    for k in ("lateral_fwhm_mm", "axial_fwhm_mm"):
        m = r.get(k)
        if m and m.get("max_rel_delta", 0.0) > max_fwhm:
            return False
    return True


def choose_mode(results: dict, modes, max_dgcnr: float = 0.01, max_fwhm: float = 0.01,
                max_fallback: float = 0.10):
    """The network-using mode with the lowest fallback rate among those that
    meet the bar within `max_fallback` (beyond it the exact solver's share of
    the frame takes most of the learned path's speed). If none does: among the
    modes with a finite gate within `max_fallback`, the one closest to the bar
    (smallest max(worst relative FWHM change / max_fwhm, worst |delta gCNR| /
    max_dgcnr), then the lower fallback rate), marked as not meeting it.
    Returns (mode, meets_bar)."""
    cands = [m for m in modes if m.use_net and m.label in results]
    ok = [m for m in cands if meets_bar(results[m.label], max_dgcnr, max_fwhm)
          and results[m.label]["fallback_rate"] <= max_fallback]
    if ok:
        return min(ok, key=lambda m: results[m.label]["fallback_rate"]), True

    def worst(m):
        r = results[m.label]
        f = max(r.get(k, {}).get("max_rel_delta", 0.0) for k in ("lateral_fwhm_mm", "axial_fwhm_mm"))
        return (max(f / max_fwhm, r.get("gcnr", {}).get("max_abs_delta", 1.0) / max_dgcnr),
                r["fallback_rate"])
    finite = [m for m in cands if (math.isfinite(m.gate) or math.isfinite(m.share) or math.isfinite(m.level))
              and results[m.label]["fallback_rate"] <= max_fallback]
    pool = finite or cands
    return (min(pool, key=worst), False) if pool else (None, False)


def at_bar_mode(results: dict, modes, max_dgcnr: float = 0.01, max_fwhm: float = 0.01):
    """The network-using mode with the lowest fallback rate among those that
    meet the bar, whatever its fallback rate (None if none does)."""
    ok = [m for m in modes if m.use_net and m.label in results
          and meets_bar(results[m.label], max_dgcnr, max_fwhm)]
    return min(ok, key=lambda m: results[m.label]["fallback_rate"]) if ok else None


def summarize(rows) -> dict:
    def flat(key, part):
        return [v for r in rows for v in r[part][key]]
    out = {"phantoms": len(rows), "fallback_rate": float(np.mean([r["fallback_rate"] for r in rows])),
           "rel_l2_mean": float(np.mean([r["rel_l2"] for r in rows]))}
    for k in ("gcnr", "cnr", "lateral_fwhm_mm", "axial_fwhm_mm"):
        p, l_ = np.array(flat(k, "plain")), np.array(flat(k, "learned"))
        if p.size:
            rel = np.abs(l_ - p) / np.maximum(np.abs(p), 1e-12)
            where = [(r["seed"], i) for r in rows for i in range(len(r["plain"][k]))]
            worst = [{"seed": int(where[j][0]), "target": int(where[j][1]), "plain": float(p[j]),
                      "learned": float(l_[j])} for j in np.argsort(-rel)[:3]]
            out[k] = {"plain_mean": float(p.mean()), "learned_mean": float(l_.mean()),
                      "max_abs_delta": float(np.max(np.abs(l_ - p))), "mean_delta": float(np.mean(l_ - p)),
                      "max_rel_delta": float(np.max(rel)), "median_rel_delta": float(np.median(rel)),
                      "n": int(p.size), "worst": worst}
    out["rows"] = rows
    return out


def load_mlp(ctx: capi.Context, path=DEFAULT_WEIGHTS) -> capi.Mlp:
    dims, params = load_weights(path)
    mlp = capi.Mlp(ctx, dims)
    mlp.set_params(params)
    return mlp


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m usx.learned")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--phantoms", type=int, default=200)
    t.add_argument("--per-phantom", type=int, default=16384)
    t.add_argument("--steps", type=int, default=50000)
    t.add_argument("--batch", type=int, default=4096)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--loss", default="subspace", choices=["output", "mse", "subspace"])
    t.add_argument("--beta", type=float, default=0.02)
    t.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    t.add_argument("--eval-phantoms", type=int, default=16)
    e = sub.add_parser("evaluate")
    e.add_argument("--weights", default=str(DEFAULT_WEIGHTS))
    e.add_argument("--phantoms", type=int, default=16)
    for p in (t, e):
        p.add_argument("--gates", default="0.1,0.3,inf",
                       help="gates on the network's distortionless residual (share gate off)")
        p.add_argument("--shares", default="0.02,0.05,0.1,0.2,0.3,0.5",
                       help="gates on the network direction's share of the power reduction (residual gate off)")
        p.add_argument("--levels", default="3,10,30,100",
                       help="gates on tr(R) over its depth's level, each alone and with every --level-shares")
        p.add_argument("--level-shares", default="inf,0.2",
                       help="share gates combined with each level gate")
        p.add_argument("--windows", default="0x0",
                       help="level-gate neighbourhoods, +/- lines x +/- depths, combined with each level gate")
        p.add_argument("--refine", type=int, default=None,
                       help="DFT beams beside the network's direction (-1: no refinement; default: "
                            "the refinement recorded with the weights when evaluating, else 4)")
        p.add_argument("--report", default=None, help="JSON report (default: beside the weights)")
    a = ap.parse_args(argv)
    if a.refine is None:
        a.refine = DEFAULT_REFINE
        if a.cmd == "evaluate" and Path(a.weights).with_suffix(".json").exists():
            recorded = trained_refine(a.weights)
            a.refine = recorded if recorded >= 0 else DEFAULT_REFINE
    sub = a.refine >= 0
    modes = modes_for([float(g) for g in a.gates.split(",") if g],
                      [float(x) for x in a.shares.split(",") if x] if sub else [], ablation=sub,
                      levels=[float(v) for v in a.levels.split(",") if v] if sub else [],
                      level_shares=[float(x) for x in a.level_shares.split(",") if x],
                      windows=[tuple(int(v) for v in w.split("x")) for w in a.windows.split(",") if w])
    imager = Imager()
    report = {"dims": list(DIMS), "setup": imager.setup.__dict__}
    eval_seeds = np.arange(900_000, 900_000 + (a.eval_phantoms if a.cmd == "train" else a.phantoms))
    if a.cmd == "train":
        train_seeds = np.arange(1000, 1000 + a.phantoms)
        t0 = time.time()
        X, T, M = make_pairs(imager, train_seeds, a.per_phantom)
        report.update(phantoms=a.phantoms, pairs=int(X.shape[0]), pair_seconds=time.time() - t0)
        Xv, Tv, Mv = make_pairs(imager, np.arange(5000, 5008), a.per_phantom, log=None)
        t0 = time.time()
        mlp, losses = train(imager.ctx, X, T, M, a.steps, a.batch, a.lr, a.seed, loss=a.loss, beta=a.beta)
        imager.ctx.synchronize()
        report.update(steps=a.steps, batch=a.batch, lr=a.lr, loss=a.loss, beta=a.beta,
                      train_seconds=time.time() - t0, losses=losses,
                      validation_loss=validation_loss(mlp, Xv, Tv, Mv))
        del X, T, M, Xv, Tv, Mv
        out = Path(a.out)
        out.parent.mkdir(parents=True, exist_ok=True)
        save_weights(out, DIMS, mlp.get_params())
    else:
        out = Path(a.weights)
        mlp = load_mlp(imager.ctx, out)
        prev = out.with_suffix(".json")
        if prev.exists():  # keep the training record, replace the evaluation
            report = {**json.loads(prev.read_text()), **report}
    results = evaluate(imager, mlp, eval_seeds, modes, refine=a.refine)
    report["refine"] = a.refine
    report["eval"] = {label: {k: v for k, v in r.items() if k != "rows"} for label, r in results.items()}
    chosen, ok = choose_mode(results, modes)
    report.pop("share_gate", None)
    report.pop("level_gate", None)
    report.pop("level_window", None)
    report.pop("at_bar", None)
    if chosen is not None:
        report.update(gate=chosen.gate, share_gate=chosen.share, level_gate=chosen.level,
                      level_window=list(chosen.window), chosen=chosen.label, meets_bar=ok)
    bar = at_bar_mode(results, modes)
    if bar is not None:
        # The setting that meets the bar at the lowest fallback, whatever that
        # costs (recorded beside the chosen one).
        report["at_bar"] = {"label": bar.label, "gate": bar.gate, "share_gate": bar.share,
                            "level_gate": bar.level, "level_window": list(bar.window),
                            "fallback_rate": results[bar.label]["fallback_rate"]}
    path = Path(a.report) if a.report else out.with_suffix(".json")
    path.write_text(json.dumps(report, indent=1, default=float))
    if chosen is not None:
        out.with_suffix(".gate").write_text(
            f"{chosen.gate} {a.refine} {chosen.share} {chosen.level} {chosen.window[0]} {chosen.window[1]}\n")
    print(json.dumps({"chosen": report.get("chosen"), "meets_bar": ok, "eval": report["eval"]}, default=float))
    imager.close()


def trained_gate(weights=DEFAULT_WEIGHTS) -> float:
    """The gate chosen when the weights were evaluated (their JSON report)."""
    p = Path(weights).with_suffix(".json")
    if p.exists():
        g = json.loads(p.read_text()).get("gate")
        if g is not None:
            return float(g)
    return DEFAULT_GATE


def trained_share_gate(weights=DEFAULT_WEIGHTS) -> float:
    """The gate on the network direction's share chosen with the weights (+inf: none)."""
    p = Path(weights).with_suffix(".json")
    if p.exists():
        g = json.loads(p.read_text()).get("share_gate")
        if g is not None:
            return float(g)
    return math.inf


def trained_level_gate(weights=DEFAULT_WEIGHTS) -> float:
    """The gate on tr(R) over its depth's level chosen with the weights (+inf: none)."""
    p = Path(weights).with_suffix(".json")
    if p.exists():
        g = json.loads(p.read_text()).get("level_gate")
        if g is not None:
            return float(g)
    return math.inf


def trained_level_window(weights=DEFAULT_WEIGHTS) -> tuple:
    """The level gate's neighbourhood chosen with the weights ((0, 0): the pixel itself)."""
    p = Path(weights).with_suffix(".json")
    if p.exists():
        w = json.loads(p.read_text()).get("level_window")
        if w is not None:
            return int(w[0]), int(w[1])
    return 0, 0


def trained_refine(weights=DEFAULT_WEIGHTS) -> int:
    """The refinement the weights were evaluated with (their JSON report)."""
    p = Path(weights).with_suffix(".json")
    if p.exists():
        r = json.loads(p.read_text()).get("refine")
        if r is not None:
            return int(r)
    return -1


if __name__ == "__main__":
    main()
