"""Learned surrogate for module expectations (C3/C4 of the benchmark plan).

* ``pair_features`` / ``sample_pairs``: source-module geometry (distance
  log-uniform on [5, 300] m, module direction and emitter direction uniform on
  the sphere) and its 8 input features.
* ``generate_tables``: one Monte-Carlo run per pair with the propagation
  kernel in histogram mode: expected hits (absorption-weighted) and a 64-bin
  histogram of log10(t_res + 21 ns) over residual times [-20, 2000] ns, with
  t_res = t - (d - r) / v_group(800 nm) as the reference's calc_time_residual!
  (src/calc.jl) defines it.
* ``MLP``: the network of csrc/pp_mlp.cu (BF16 tcgen05 forward/backward,
  Adam), trained by ``train``.

There is no surrogate in the reference repository (it loads an external
PhotonSurrogateModel, examples/validation.jl:455,673-676).
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_float, c_int32, c_int64, c_void_p
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check
from .medium import CascadiaMediumProperties
from .sources import ExtendedCherenkovEmitter, LongitudinalParameterisation, to_records
from .spectrum import make_cherenkov_spectrum
from .targets import HomogeneousDetector, Spherical

N_FEATURES = 8
N_BINS = 64
T_OFFSET = 21.0                 # ns: log10(t_res + 21) maps [-20, 2000] to [0, log10 2021]
LOG_T_LO = 0.0
LOG_T_HI = float(np.log10(2021.0))
D_MIN, D_MAX = 5.0, 300.0
MODULE_RADIUS = 0.2159
CASCADE = LongitudinalParameterisation(2.0, 0.63, 0.36)


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


@dataclass
class Pairs:
    distance: np.ndarray     # m
    module_dir: np.ndarray   # unit vector source -> module
    emitter_dir: np.ndarray  # unit emitter axis
    spectrum_id: np.ndarray  # 0 = Frank-Tamm on 300-800 nm

    def __len__(self):
        return int(self.distance.shape[0])

    def subset(self, idx):
        return Pairs(self.distance[idx], self.module_dir[idx], self.emitter_dir[idx],
                     self.spectrum_id[idx])


def sample_pairs(n: int, seed: int = 0) -> Pairs:
    rng = np.random.default_rng(seed)
    d = np.exp(rng.uniform(np.log(D_MIN), np.log(D_MAX), n))
    return Pairs(d, _unit(rng, n), _unit(rng, n), np.zeros(n, np.int32))


def pair_features(p: Pairs) -> np.ndarray:
    """[log-distance (scaled), cos/sin of the emitter-to-module angle, cos/sin of
    the module azimuth about the emitter axis, cos/sin of the emitter azimuth,
    spectrum id]."""
    e, m = p.emitter_dir, p.module_dir
    ct = np.clip(np.sum(e * m, axis=1), -1.0, 1.0)
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    phi_m = np.arctan2(m[:, 1], m[:, 0])
    phi_e = np.arctan2(e[:, 1], e[:, 0])
    ld = (np.log10(p.distance) - 1.34) / 0.45
    x = np.stack([ld, ct, st, np.cos(phi_m), np.sin(phi_m), np.cos(phi_e), np.sin(phi_e),
                  p.spectrum_id.astype(np.float64)], axis=1)
    return x.astype(np.float32)


def feature_box(n_spectra: int = 1):
    """Bounds of pair_features over the training ranges: (lo, hi), 8 each."""
    ld = (np.log10([D_MIN, D_MAX]) - 1.34) / 0.45
    lo = np.array([ld[0], -1, 0, -1, -1, -1, -1, 0], np.float64)
    hi = np.array([ld[1], 1, 1, 1, 1, 1, 1, n_spectra - 1], np.float64)
    return lo, hi


# The fused inference stores hidden activations (and half pre-activations) in
# BF16, whose largest finite value is FP32's to 8 bits; a network whose
# activations could pass it would give infinities.
BF16_MAX = 3.3895313892515355e38


def _silu_interval(zl, zh):
    """Image of [zl, zh] under SiLU (decreasing below its minimum at
    z = -1.27846, increasing above)."""
    def silu(z):
        return z / (1.0 + np.exp(-np.clip(z, -80, 80)))
    z_min, v_min = -1.2784645, -0.2784645
    hi = np.maximum(silu(zl), silu(zh))
    lo = np.where(zl >= z_min, silu(zl), np.where(zh >= z_min, v_min, silu(zh)))
    return lo, hi


def activation_bound(W, b, lo, hi) -> float:
    """Largest magnitude any hidden pre-activation or activation of the network
    (W, b as MLP.unpack gives them) can reach for inputs in the box [lo, hi],
    by interval arithmetic (midpoint-radius form, exact per layer for a box).
    Below BF16_MAX, the fused inference cannot overflow for such inputs."""
    xl, xh = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    worst = float(np.max(np.abs(np.concatenate([xl, xh]))))
    for l in range(len(W) - 1):
        w = np.asarray(W[l], np.float64)[:, :xl.shape[0]]
        c, r = 0.5 * (xl + xh), 0.5 * (xh - xl)
        zc = w @ c + np.asarray(b[l], np.float64)
        zr = np.abs(w) @ r
        zl, zh = zc - zr, zc + zr
        worst = max(worst, float(np.max(np.abs(np.concatenate([zl, zh])))))
        xl, xh = _silu_interval(zl, zh)
        worst = max(worst, float(np.max(np.abs(np.concatenate([xl, xh])))))
    return worst


def in_training_range(p: Pairs) -> np.ndarray:
    return (p.distance >= D_MIN) & (p.distance <= D_MAX) & (p.spectrum_id == 0)


def source_positions(p: Pairs) -> np.ndarray:
    """Cascade vertex of each pair with the module at the origin."""
    return -p.distance[:, None] * p.module_dir


def geometric_time(p: Pairs, medium=None) -> np.ndarray:
    """(d - r) / v_group(800 nm), the direct-light time of the reference's
    calc_tgeo (src/calc.jl) for a module of radius MODULE_RADIUS."""
    medium = medium or CascadiaMediumProperties()
    return (p.distance - MODULE_RADIUS) / float(medium.group_velocity(800.0))


def cascade_records(pairs: Pairs, photons: int):
    """The pp_source records of table_setup's emitters, filled column-wise
    (the same bytes as converting each ExtendedCherenkovEmitter)."""
    n = len(pairs)
    rec = np.zeros(max(1, n), dtype=np.dtype(_lib.pp_source))
    rec["kind"][:n] = _lib.PP_SRC_EXTENDED_CHERENKOV
    rec["photons"][:n] = int(photons)
    rec["position"][:n] = source_positions(pairs).astype(np.float32)
    rec["direction"][:n] = pairs.emitter_dir.astype(np.float32)
    rec["long_a"][:n] = CASCADE.a
    rec["long_b"][:n] = CASCADE.b
    rec["long_lrad"][:n] = CASCADE.lrad
    arr = (_lib.pp_source * max(1, n)).from_buffer(rec)
    arr._keep = rec
    return arr


def table_setup(pairs: Pairs, photons: int, seed: int, medium=None, spectrum=None):
    """One PhotonPropSetup holding every pair: the module at the origin and one
    ExtendedCherenkovEmitter per pair (source index = pair index)."""
    from .propsetup import PhotonPropSetup
    medium = medium or CascadiaMediumProperties()
    spectrum = spectrum or make_cherenkov_spectrum((300.0, 800.0), medium)
    pos = source_positions(pairs)
    srcs = [ExtendedCherenkovEmitter(pos[i], pairs.emitter_dir[i], 0.0, photons, CASCADE)
            for i in range(len(pairs))]
    tgt = HomogeneousDetector(Spherical([0.0, 0.0, 0.0], MODULE_RADIUS), 1.0, 1)
    return PhotonPropSetup(srcs, [tgt], medium, spectrum, seed)


def generate_tables(pairs: Pairs, photons: int, seed: int = 1, ctx=None, medium=None,
                    spectrum=None, device: int = 0, chunk: int = 262144, n_steps: int = 15,
                    device_out: bool = False):
    """Expected hits and time histograms of every pair (one MC run each).

    The module sits at the origin; pair i is a cascade at -d_i * module_dir_i
    pointing along emitter_dir_i, so all pairs share one target and run in one
    persistent launch per chunk of pairs (chunk k uses seed + k * chunk).
    Returns (counts [n], hists [n x 64]) for `photons` photons per pair, as
    numpy arrays or, with device_out, as CUDA tensors."""
    import torch
    from .context import Context
    medium = medium or CascadiaMediumProperties()
    spectrum = spectrum or make_cherenkov_spectrum((300.0, 800.0), medium)
    own = ctx is None
    ctx = ctx or Context(device)
    n = len(pairs)
    counts = torch.empty(n, dtype=torch.float32, device="cuda")
    hists = torch.empty((n, N_BINS), dtype=torch.float32, device="cuda")
    ctr = torch.zeros(64, dtype=torch.uint8, device="cuda")
    tgeo_all = torch.tensor(geometric_time(pairs, medium), dtype=torch.float32, device="cuda")
    table_setup(pairs.subset(slice(0, 1)), photons, seed, medium, spectrum).upload(ctx)
    for lo in range(0, n, chunk):
        hi = min(n, lo + chunk)
        ctx.set_sources(cascade_records(pairs.subset(slice(lo, hi)), photons), hi - lo, 1.0)
        hist = torch.empty((hi - lo, N_BINS + 1), dtype=torch.float32, device="cuda")
        check(ctx._lib.pp_launch_histogram(ctx.ptr, seed + lo, n_steps,
                                           c_void_p(tgeo_all[lo:hi].data_ptr()),
                                           c_void_p(hist.data_ptr()), N_BINS, T_OFFSET, LOG_T_LO,
                                           LOG_T_HI, c_void_p(ctr.data_ptr()), None),
              "pp_launch_histogram")
        counts[lo:hi] = hist[:, 0]
        hists[lo:hi] = hist[:, 1:]
    torch.cuda.synchronize()
    if own:
        ctx.close()
    if device_out:
        return counts, hists
    return counts.cpu().numpy(), hists.cpu().numpy()


class MLP:
    """Handle on a pp_mlp (parameters and optimiser state live on the device)."""

    def __init__(self, device=0, n_in=N_FEATURES, hidden=256, n_layers=4, n_bins=N_BINS,
                 max_batch=8192, seed=0):
        self._lib = _lib.load()
        p = c_void_p()
        check(self._lib.pp_mlp_create(byref(p), device, n_in, hidden, n_layers, n_bins,
                                      max_batch, seed), "pp_mlp_create")
        self.ptr = p
        self.n_in, self.hidden, self.n_layers, self.n_bins = n_in, hidden, n_layers, n_bins
        self.max_batch = max_batch
        n = c_int64()
        check(self._lib.pp_mlp_num_params(self.ptr, byref(n)))
        self.n_params = n.value

    def close(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._lib.pp_mlp_destroy(self.ptr)
            self.ptr = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layout(self, layer):
        ow, ob, r, c = c_int64(), c_int64(), c_int32(), c_int32()
        check(self._lib.pp_mlp_layout(self.ptr, layer, byref(ow), byref(ob), byref(r), byref(c)))
        return ow.value, ob.value, r.value, c.value

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        check(self._lib.pp_mlp_get_params(self.ptr, out.ctypes.data_as(ctypes.POINTER(c_float)),
                                          self.n_params))
        return out

    def set_params(self, v: np.ndarray) -> None:
        v = np.ascontiguousarray(v, np.float32)
        check(self._lib.pp_mlp_set_params(self.ptr, v.ctypes.data_as(ctypes.POINTER(c_float)),
                                          self.n_params))

    def activation_bound(self, lo=None, hi=None) -> float:
        """activation_bound of the current parameters over an input box (by
        default the training features' box)."""
        if lo is None:
            lo, hi = feature_box()
        W, b = self.unpack(self.params())
        return activation_bound(W, b, lo, hi)

    def unpack(self, flat):
        W, b = [], []
        for l in range(self.n_layers + 1):
            ow, ob, r, c = self.layout(l)
            W.append(flat[ow:ow + r * c].reshape(r, c))
            b.append(flat[ob:ob + r])
        return W, b

    def forward(self, x_dev, B, out_dev, stream=0):
        check(self._lib.pp_mlp_forward(self.ptr, c_void_p(x_dev), B, c_void_p(out_dev),
                                       c_void_p(stream)), "pp_mlp_forward")

    def infer(self, x_dev, n, expect_dev, pdf_dev=0, stream=0, check_now=True):
        """Fused tcgen05 inference of n rows (device pointers): expected counts
        and, when pdf_dev is given, the time PDFs (n x n_bins)."""
        check(self._lib.pp_mlp_infer(self.ptr, c_void_p(x_dev), int(n), c_void_p(expect_dev),
                                     c_void_p(pdf_dev or None), c_void_p(stream)), "pp_mlp_infer")
        if check_now:
            check(self._lib.pp_mlp_check(self.ptr, c_void_p(stream)), "pp_mlp_infer")

    def loss_grad(self, x_dev, count_dev, hist_dev, B):
        g = np.empty(self.n_params, np.float32)
        loss = c_float()
        check(self._lib.pp_mlp_loss_grad(self.ptr, c_void_p(x_dev), c_void_p(count_dev),
                                         c_void_p(hist_dev), B,
                                         g.ctypes.data_as(ctypes.POINTER(c_float)), byref(loss),
                                         None), "pp_mlp_loss_grad")
        return loss.value, g

    def train_step(self, x_dev, count_dev, hist_dev, B, lr, stream=0):
        check(self._lib.pp_mlp_train_step(self.ptr, c_void_p(x_dev), c_void_p(count_dev),
                                          c_void_p(hist_dev), B, float(lr), c_void_p(stream)),
              "pp_mlp_train_step")

    def train_steps(self, x_dev, count_dev, hist_dev, n_rows, B, n_steps, step0, total, lr0,
                    lr1, seed, stream=0):
        """`n_steps` Adam steps inside the library (pp_mlp_train_steps): batches
        of `B` rows drawn on the device from the `n_rows` training rows, cosine
        step size from `lr0` to `lr1` over `total` steps begun at Adam step
        `step0`, one captured step replayed per step."""
        check(self._lib.pp_mlp_train_steps(self.ptr, c_void_p(x_dev), c_void_p(count_dev),
                                           c_void_p(hist_dev), int(n_rows), int(B), int(n_steps),
                                           int(step0), int(total), float(lr0), float(lr1),
                                           int(seed) & (2**64 - 1), c_void_p(stream)),
              "pp_mlp_train_steps")

    def step_count(self) -> int:
        """Adam steps taken so far."""
        v = c_int64()
        check(self._lib.pp_mlp_step_count(self.ptr, byref(v)), "pp_mlp_step_count")
        return v.value

    def save(self, path: str) -> None:
        """Checkpoint: shape, parameters and Adam state in one .npz file."""
        m = np.empty(self.n_params, np.float32)
        v = np.empty(self.n_params, np.float32)
        st = c_int64()
        fp = ctypes.POINTER(c_float)
        check(self._lib.pp_mlp_get_adam(self.ptr, m.ctypes.data_as(fp), v.ctypes.data_as(fp),
                                        self.n_params, byref(st)), "pp_mlp_get_adam")
        np.savez(path, shape=np.array([self.n_in, self.hidden, self.n_layers, self.n_bins]),
                 params=self.params(), adam_m=m, adam_v=v, step=np.array([st.value]))

    @classmethod
    def load(cls, path: str, device=0, max_batch=8192):
        z = np.load(path)
        n_in, hidden, n_layers, n_bins = (int(v) for v in z["shape"])
        net = cls(device=device, n_in=n_in, hidden=hidden, n_layers=n_layers, n_bins=n_bins,
                  max_batch=max_batch)
        net.set_params(z["params"])
        fp = ctypes.POINTER(c_float)
        m = np.ascontiguousarray(z["adam_m"], np.float32)
        v = np.ascontiguousarray(z["adam_v"], np.float32)
        check(net._lib.pp_mlp_set_adam(net.ptr, m.ctypes.data_as(fp), v.ctypes.data_as(fp),
                                       net.n_params, int(z["step"][0])), "pp_mlp_set_adam")
        return net

    def last_loss(self) -> float:
        v = c_float()
        check(self._lib.pp_mlp_last_loss(self.ptr, byref(v)), "pp_mlp_last_loss")
        return v.value


def train(mlp: MLP, x, counts, hists, steps: int, batch: int = 8192, lr: float = 1e-3,
          seed: int = 0, log_every: int = 0, lr_final: float | None = None, stream: int = 0):
    """Adam on (features, expected hits, time histograms) held in device memory
    (torch tensors, float32, contiguous); returns the list of (step, loss)
    logged every `log_every` steps and at the last.  The step size starts at
    `lr` and follows a cosine down to `lr_final` (default lr / 100) at the last
    step, so that the final parameters are not those of one noisy step at full
    rate.  Batches are drawn on the device (Philox, keyed on `seed` and the Adam
    step), and the steps between two log points run as replays of one captured
    step, without a return to Python."""
    lr_final = lr * 0.01 if lr_final is None else lr_final
    x, counts, hists = (t.contiguous().float() for t in (x, counts, hists))
    n = x.shape[0]
    step0 = mlp.step_count()
    points = sorted({s for s in range(0, steps, log_every)} | {steps - 1}) if log_every \
        else [steps - 1]
    log, done = [], 0
    for p in points:
        if p < 0:
            continue
        mlp.train_steps(x.data_ptr(), counts.data_ptr(), hists.data_ptr(), n, batch, p + 1 - done,
                        step0, steps, lr, lr_final, seed, stream)
        done = p + 1
        if log_every:
            log.append((p, mlp.last_loss()))
    return log


# ---------------------------------------------------------------------------
# Serving: the network answers, the plain MC is fallback and judge.

def analytic_expectation(p: Pairs, photons: float, att_len: float = 25.0,
                         norm: float = 1.0) -> np.ndarray:
    """The reference's closed-form distance scaling of a module's photon
    count, norm * N * r^2 / (4 d^2) * exp(-d / att_len)
    (examples/validation.jl:307-312): the method without a surrogate."""
    return norm * photons * MODULE_RADIUS ** 2 / (4.0 * p.distance ** 2) * np.exp(
        -p.distance / att_len)


def fit_analytic_norm(p: Pairs, counts: np.ndarray, photons: float, att_len: float = 25.0):
    """Least-squares norm of analytic_expectation to MC counts (the
    curve_fit of examples/validation.jl:314)."""
    a = analytic_expectation(p, photons, att_len)
    return float(np.sum(a * counts) / max(np.sum(a * a), 1e-300))


def ks_distance(pdf: np.ndarray, hist: np.ndarray) -> np.ndarray:
    """Row-wise Kolmogorov-Smirnov distance between binned PDFs and histograms."""
    c1 = np.cumsum(pdf, axis=1)
    c1 = c1 / np.maximum(c1[:, -1:], 1e-30)
    c2 = np.cumsum(hist, axis=1)
    c2 = c2 / np.maximum(c2[:, -1:], 1e-30)
    return np.abs(c1 - c2).max(axis=1)


@dataclass
class Expectations:
    counts: np.ndarray          # expected hits for the requested photons per pair
    pdf: np.ndarray | None      # n x N_BINS arrival-time PDFs (None if not requested;
                                # NaN rows: answered by an MC run that saw no hit)
    from_mc: np.ndarray         # bool: answered by the MC (outside range, audited, failed)
    audit: dict                 # audit statistics of this batch


def calibration(pred, obs, n_groups: int = 10) -> dict:
    """Calibration of predicted against observed counts over ALL pairs (dim
    ones included): the pairs are split into n_groups equal groups by
    predicted count; per group the sums of both, the relative bias
    sum(obs) / sum(pred) - 1 and the pull (sum(obs) - sum(pred)) /
    sqrt(sum(pred)).  The MC counts are sums of absorption weights w <= 1, whose
    variance sum(w^2) is at most the Poisson sum(w), so these pulls are
    conservative (too small by at most that factor); they ignore the network's
    own spread."""
    pred = np.asarray(pred, np.float64)
    obs = np.asarray(obs, np.float64)
    order = np.argsort(pred, kind="stable")
    groups = []
    for g in np.array_split(order, n_groups):
        if g.size == 0:
            continue
        sp, so = float(pred[g].sum()), float(obs[g].sum())
        groups.append({"n": int(g.size), "pred_lo": float(pred[g].min()),
                       "pred_hi": float(pred[g].max()), "sum_pred": sp, "sum_obs": so,
                       "rel_bias": so / sp - 1.0 if sp > 0 else float("nan"),
                       "pull": (so - sp) / np.sqrt(sp) if sp > 0 else float("nan")})
    pulls = [g["pull"] for g in groups if np.isfinite(g["pull"])]
    biases = [g["rel_bias"] for g in groups if np.isfinite(g["rel_bias"])]
    return {"groups": groups, "max_abs_pull": float(np.max(np.abs(pulls))) if pulls else None,
            "max_abs_rel_bias": float(np.max(np.abs(biases))) if biases else None,
            "total_rel_bias": float(obs.sum() / pred.sum() - 1.0) if pred.sum() > 0 else None}


class Surrogate:
    """Module expectations from the trained network, with the plain MC as
    fallback and judge.

    Pairs outside the training ranges, and a random `audit_fraction` of the
    rest, run through the MC at `fallback_photons` per pair.  The audited
    pairs measure the network's error on this batch: relative count error
    where the MC saw at least `min_audit_hits` (so that its own Poisson error
    is small), the KS distance of the time PDFs, and the calibration of the
    counts over every audited pair (deciles of the predicted count, see
    `calibration`).  The network answers only pairs inside the training
    ranges, whose features lie in `feature_box()`; if the network's
    `activation_bound` over that box reaches BF16_MAX (the fused kernel's
    BF16 activations could overflow), the batch fails its
    check as well.  If the median count
    error exceeds `max_median_error`, the batch fails its error check and,
    with on_failure="mc", every pair of the batch is answered by the MC."""

    def __init__(self, mlp: MLP, table_photons: float = 1e5, ctx=None,
                 fallback_photons: int = 10_000_000, audit_fraction: float = 0.01,
                 min_audit_hits: float = 400.0, max_median_error: float = 0.05,
                 on_failure: str = "mc", medium=None, spectrum=None):
        if on_failure not in ("mc", "flag"):
            raise ValueError("on_failure must be 'mc' or 'flag'")
        self.mlp = mlp
        self.table_photons = float(table_photons)
        self.ctx = ctx
        self.fallback_photons = int(fallback_photons)
        self.audit_fraction = float(audit_fraction)
        self.min_audit_hits = float(min_audit_hits)
        self.max_median_error = float(max_median_error)
        self.on_failure = on_failure
        self.medium = medium
        self.spectrum = spectrum

    def infer(self, p: Pairs, with_pdf: bool = True):
        """Network outputs for every pair (device tensors: counts per
        table_photons, PDFs or None)."""
        import torch
        n = len(p)
        x = torch.tensor(pair_features(p), device="cuda")
        counts = torch.empty(n, dtype=torch.float32, device="cuda")
        pdf = torch.empty((n, N_BINS), dtype=torch.float32, device="cuda") if with_pdf else None
        self.mlp.infer(x.data_ptr(), n, counts.data_ptr(), pdf.data_ptr() if with_pdf else 0)
        return counts, pdf

    @staticmethod
    def _normalise(h):
        """Histograms to PDFs; rows without any MC hit have no PDF (NaN)."""
        tot = h.sum(axis=1, keepdims=True)
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.where(tot > 0, h / tot, np.nan)

    def _mc(self, p: Pairs, seed: int):
        if self.spectrum is None and np.any(p.spectrum_id != 0):
            raise ValueError("only spectrum id 0 (Frank-Tamm, 300-800 nm) has a default table")
        c, h = generate_tables(p, self.fallback_photons, seed=seed, ctx=self.ctx,
                               medium=self.medium, spectrum=self.spectrum)
        return c.astype(np.float64), h

    def expectations(self, p: Pairs, photons: float | None = None, seed: int = 0,
                     with_pdf: bool = True) -> Expectations:
        import time
        photons = self.table_photons if photons is None else float(photons)
        n = len(p)
        t0 = time.perf_counter()
        counts_d, pdf_d = self.infer(p, with_pdf)
        counts = counts_d.cpu().numpy().astype(np.float64) * (photons / self.table_photons)
        pdf = pdf_d.cpu().numpy() if with_pdf else None
        t_nn = time.perf_counter() - t0
        rng = np.random.default_rng(seed)
        inside = in_training_range(p)
        audit = np.flatnonzero(inside & (rng.random(n) < self.audit_fraction))
        mc_idx = np.union1d(np.flatnonzero(~inside), audit)
        from_mc = np.zeros(n, bool)
        stats = {"n_pairs": n, "n_outside": int((~inside).sum()), "n_audited": int(audit.size),
                 "nn_seconds": t_nn, "mc_pairs": int(mc_idx.size), "mc_seconds": 0.0}
        if mc_idx.size:
            t0 = time.perf_counter()
            mc_c, mc_h = self._mc(p.subset(mc_idx), seed)
            stats["mc_seconds"] = time.perf_counter() - t0
            scale = photons / self.fallback_photons
            pos = np.searchsorted(mc_idx, audit)
            judged = mc_c[pos] >= self.min_audit_hits
            nn_a = counts[audit] / scale
            if audit.size:
                stats["calibration"] = calibration(nn_a, mc_c[pos])
            rel = np.abs(nn_a[judged] - mc_c[pos][judged]) / mc_c[pos][judged]
            stats.update({
                "n_judged": int(judged.sum()),
                "median_rel_error": float(np.median(rel)) if rel.size else float("nan"),
                "p95_rel_error": float(np.quantile(rel, 0.95)) if rel.size else float("nan"),
                # the part of the error that is the judge's own Poisson noise
                "judge_noise_median": float(np.median(0.6745 / np.sqrt(mc_c[pos][judged])))
                if rel.size else float("nan"),
            })
            if with_pdf and rel.size:
                ks = ks_distance(pdf[audit][judged], mc_h[pos][judged])
                stats.update({"median_ks": float(np.median(ks)),
                              "p95_ks": float(np.quantile(ks, 0.95))})
            counts[mc_idx] = mc_c * scale
            if with_pdf:
                pdf[mc_idx] = self._normalise(mc_h)
            from_mc[mc_idx] = True
        bound = self.mlp.activation_bound()
        stats["activation_bound"] = bound
        # no audited pair with enough MC statistics: no evidence against the network
        failed = bool(stats.get("median_rel_error", 0.0) > self.max_median_error
                      or not bound < BF16_MAX)
        stats["passed"] = not failed
        if failed and self.on_failure == "mc":
            rest = np.flatnonzero(~from_mc)
            if rest.size:
                t0 = time.perf_counter()
                mc_c, mc_h = self._mc(p.subset(rest), seed + 1)
                stats["mc_seconds"] += time.perf_counter() - t0
                stats["mc_pairs"] += int(rest.size)
                counts[rest] = mc_c * (photons / self.fallback_photons)
                if with_pdf:
                    pdf[rest] = self._normalise(mc_h)
                from_mc[rest] = True
        return Expectations(counts, pdf, from_mc, stats)


# ---------------------------------------------------------------------------
# Table files.

class TableStore:
    """Append-only store of surrogate tables: a directory of parts
    ``part_00001.npz``, ``part_00002.npz``, ... each holding one batch of pairs
    (distance, module_dir, emitter_dir, spectrum_id), their counts and
    histograms, and the batch's attributes (photons, seed, ...).  The
    append-with-counter pattern of the reference's save_hdf! (group,
    dataset_k, nsims; scripts/photon_tables/utils.jl:24-56) -- without HDF5,
    which needs h5py, absent here -- so a table run can be resumed batch by
    batch (generate_tables is deterministic per batch and seed)."""

    def __init__(self, path: str):
        import os
        self.path = path
        os.makedirs(path, exist_ok=True)

    @property
    def nsims(self) -> int:
        import os
        return sum(1 for f in os.listdir(self.path) if f.startswith("part_") and f.endswith(".npz"))

    def append(self, pairs: Pairs, counts, hists, **attrs) -> str:
        import json
        import os
        k = self.nsims + 1
        fname = os.path.join(self.path, f"part_{k:05d}.npz")
        np.savez(fname, distance=pairs.distance, module_dir=pairs.module_dir,
                 emitter_dir=pairs.emitter_dir, spectrum_id=pairs.spectrum_id,
                 counts=np.asarray(counts, np.float32), hists=np.asarray(hists, np.float32),
                 attrs=np.array(json.dumps(attrs)))
        return fname

    def read(self):
        """(Pairs, counts, hists, [attrs per part]) of all parts in order."""
        import json
        import os
        parts = sorted(f for f in os.listdir(self.path) if f.startswith("part_"))
        zs = [np.load(os.path.join(self.path, f)) for f in parts]
        if not zs:
            return Pairs(np.zeros(0), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0, np.int32)), \
                np.zeros(0, np.float32), np.zeros((0, N_BINS), np.float32), []
        cat = lambda k: np.concatenate([z[k] for z in zs])  # noqa: E731
        pairs = Pairs(cat("distance"), cat("module_dir"), cat("emitter_dir"), cat("spectrum_id"))
        return pairs, cat("counts"), cat("hists"), [json.loads(str(z["attrs"])) for z in zs]


def write_arrow(path: str, pairs: Pairs, counts, hists, **attrs) -> None:
    """Arrow IPC file of a table (one row per pair: distance, module and
    emitter directions, spectrum id, count, histogram; attributes in the
    schema metadata), the format of the reference's photon_table_for_sr.jl
    writer (scripts/photon_tables/photon_table_for_sr.jl:214-224).  Needs
    pyarrow."""
    import json

    import pyarrow as pa
    n = len(pairs)
    cols = {
        "distance": pa.array(pairs.distance, pa.float64()),
        "module_dir": pa.FixedSizeListArray.from_arrays(
            pa.array(np.asarray(pairs.module_dir, np.float64).ravel()), 3),
        "emitter_dir": pa.FixedSizeListArray.from_arrays(
            pa.array(np.asarray(pairs.emitter_dir, np.float64).ravel()), 3),
        "spectrum_id": pa.array(np.asarray(pairs.spectrum_id, np.int32)),
        "count": pa.array(np.asarray(counts, np.float32)),
        "hist": pa.FixedSizeListArray.from_arrays(
            pa.array(np.asarray(hists, np.float32).reshape(n, -1).ravel()),
            np.asarray(hists).shape[1] if n else N_BINS),
    }
    table = pa.table(cols).replace_schema_metadata({"attrs": json.dumps(attrs)})
    with pa.OSFile(path, "wb") as f, pa.ipc.new_file(f, table.schema) as w:
        w.write_table(table)


def read_arrow(path: str):
    """(Pairs, counts, hists, attrs) of a write_arrow file."""
    import json

    import pyarrow as pa
    with pa.memory_map(path) as f:
        table = pa.ipc.open_file(f).read_all()
    n = table.num_rows
    flat = lambda name, w: np.asarray(table.column(name).combine_chunks().flatten()).reshape(n, w)  # noqa: E731
    pairs = Pairs(np.asarray(table.column("distance")), flat("module_dir", 3),
                  flat("emitter_dir", 3), np.asarray(table.column("spectrum_id")))
    hists = flat("hist", table.schema.field("hist").type.list_size)
    attrs = json.loads(table.schema.metadata[b"attrs"].decode())
    return pairs, np.asarray(table.column("count")), hists, attrs
