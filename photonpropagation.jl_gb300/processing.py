"""propagate_photons and its helpers (mirrors src/processing.jl:32-75 and
src/photon_prop_cuda.jl:878-959)."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _lib
from .context import Context, device_memory
from .targets import module_ids

_CONTEXTS: dict = {}


class PhotonPropOOMException(Exception):
    """The hit buffer was too small (src/photon_prop_cuda.jl:40, :937-939)."""


@dataclass
class PhotonHit:
    """One row of the hit table (PhotonHit, src/photon_prop_cuda.jl:407-416),
    for code that walks hits one by one; ``HitTable.rows()`` yields them."""
    position: np.ndarray
    direction: np.ndarray
    initial_direction: np.ndarray
    wavelength: float
    time: float
    dist_travelled: float
    module_id: int
    n_steps: int


class HitTable(dict):
    """Column table of hits (the reference returns a DataFrame with these
    columns; numpy arrays keyed by column name here)."""

    @property
    def nrow(self) -> int:
        return int(self["wavelength"].shape[0]) if "wavelength" in self else 0

    def rows(self):
        for i in range(self.nrow):
            yield PhotonHit(self["position"][i], self["direction"][i],
                            self["initial_direction"][i], float(self["wavelength"][i]),
                            float(self["time"][i]), float(self["dist_travelled"][i]),
                            int(self["module_id"][i]), int(self["n_steps"][i]))


class HitBuffers:
    """Capacity of the hit buffer (make_hit_buffers, src/photon_prop_cuda.jl:878-886).

    The reference allocates ``reserved_memory_fraction * totalmem / sizeof(hit)``
    records on the device and on the host; here only the device buffer is held
    (by the context), sized min(capacity, photons), and the host receives just
    the rows that were hit."""

    def __init__(self, capacity: int, device: int = 0):
        self.capacity = int(capacity)
        self.device = device


def make_hit_buffers(time_type=np.float64, reserved_memory_fraction: float = 0.7,
                     device: int = 0) -> HitBuffers:
    _, total = device_memory(device)
    rec = 80  # bytes per pp_hit_record
    return HitBuffers(int(reserved_memory_fraction * total) // rec, device)


def get_context(device: int = 0) -> Context:
    ctx = _CONTEXTS.get(device)
    if ctx is None:
        ctx = Context(device)
        _CONTEXTS[device] = ctx
    return ctx


def _ensure_uploaded(setup, ctx) -> None:
    """Upload the setup's device inputs unless the context already holds them
    (the context records what its last PhotonPropSetup.upload sent; any other
    setter clears the record)."""
    if not setup.is_uploaded(ctx):
        setup.upload(ctx)


def _run(setup, hit_buffers: HitBuffers, n_steps: int):
    ctx = get_context(hit_buffers.device)
    _ensure_uploaded(setup, ctx)
    recs = setup.source_records()
    rc, n_hits, n_ph_sim = ctx.propagate(recs, len(setup.sources), setup.seed, n_steps,
                                         setup.photon_scaling, hit_buffers.capacity)
    if rc == _lib.PP_ERR_OVERFLOW:
        raise PhotonPropOOMException(
            f"{n_hits} hits exceed the hit buffer capacity {hit_buffers.capacity}")
    return ctx.fetch_hits(n_hits), n_ph_sim


def autotune(setup, steps: int = 15, sample_photons: int = 8_000_000, device: int = 0) -> dict:
    """Choose the launch shape (threads per block, photons per thread) and the
    grid and safety-field cell sizes for `setup` by timing candidate
    configurations on a photon sample (``pp_autotune``), and keep them on the
    device's context: later ``propagate_photons`` calls on that device (any
    setup) run with them.  The reference has no counterpart; its launch shape
    is fixed.  Returns the chosen tuning and the sample's photons/s."""
    ctx = get_context(device)
    _ensure_uploaded(setup, ctx)
    recs = setup.source_records()
    ctx.set_sources(recs, len(setup.sources), setup.photon_scaling)
    t, rate = ctx.autotune(setup.seed, steps, sample_photons=sample_photons)
    return dict(block_threads=t.block_threads, photons_per_thread=t.photons_per_thread,
                cell_size=t.cell_size, safety_cell=t.safety_cell, photons_per_s=rate)


def run_photon_prop_no_local_cache(sources, targets, medium, spectrum, seed,
                                   hit_buffers: HitBuffers, n_steps: int = 15,
                                   photon_scaling: float = 1.0):
    """Propagate `sources` to `targets`; returns (hit columns, n_ph_sim)
    (src/photon_prop_cuda.jl:889-959).  The columns hold module_index (1-based
    target index) as the reference kernel does.  Raises PhotonPropOOMException
    when the hits exceed the buffer capacity."""
    from .propsetup import PhotonPropSetup
    setup = PhotonPropSetup(sources, targets, medium, spectrum, seed,
                            photon_scaling=photon_scaling)
    return _run(setup, hit_buffers, n_steps)


def calc_total_weight(table: HitTable, setup) -> HitTable:
    """abs_weight = exp(-dist / abs_len(wl)) in FP64 and total_weight =
    base_weight * abs_weight (src/processing.jl:32-44), recomputed on the host."""
    if table.nrow == 0:
        return table
    abs_len = np.asarray(setup.medium.absorption_length(table["wavelength"].astype(np.float64)),
                         np.float32)
    ratio = (table["dist_travelled"].astype(np.float32) / abs_len).astype(np.float64)
    table["abs_weight"] = np.exp(-ratio)
    table["total_weight"] = table["base_weight"] * table["abs_weight"]
    return table


def propagate_photons(setup, *buffers, steps: int = 15, reserved_memory_fraction: float = 0.7,
                      copy_output: bool = False, device: int = 0) -> HitTable:
    """``propagate_photons(setup, steps=15; reserved_memory_fraction=0.7)`` and
    ``propagate_photons(setup, hit_buffers, steps=15)`` (src/processing.jl:47-75).

    Returns the hit table with columns position, direction, initial_direction,
    wavelength, time, dist_travelled, module_id, n_steps, base_weight,
    abs_weight (computed in the kernel), total_weight, plus photon_index and
    source_index."""
    hb = None
    rest = list(buffers)
    if rest and isinstance(rest[0], HitBuffers):
        hb = rest.pop(0)
        if rest and isinstance(rest[0], HitBuffers):  # (hbc, hbg) pair as in the reference
            rest.pop(0)
    if rest:
        steps = int(rest.pop(0))
    ids = module_ids(setup.targets)  # raises for DetectorLines, as the reference does
    if hb is None:
        hb = make_hit_buffers(reserved_memory_fraction=reserved_memory_fraction, device=device)
    cols, n_ph_sim = _run(setup, hb, steps)
    t = HitTable()
    n = cols["wavelength"].shape[0]
    for k in ("position", "direction", "initial_direction", "wavelength", "time",
              "dist_travelled"):
        t[k] = cols[k]
    t["module_id"] = ids[cols["module_index"] - 1] if n else np.zeros(0, np.uint16)
    t["n_steps"] = cols["n_steps"]
    total = sum(int(s.photons) for s in setup.sources)
    base = total / n_ph_sim if n_ph_sim > 0 else float("inf")
    t["base_weight"] = np.full(n, base, np.float64)
    t["abs_weight"] = cols["abs_weight"].astype(np.float64)
    t["total_weight"] = t["base_weight"] * t["abs_weight"]
    t["photon_index"] = cols["photon_index"]
    t["source_index"] = cols["source_index"]
    t.n_ph_sim = n_ph_sim
    return t


def calc_number_of_steps(sca_len: float, cutoff_distance: float, percentile: float = 0.9) -> int:
    """``calc_number_of_steps`` (src/processing.jl:154-177): the smallest n from
    ceil(cutoff / sca_len) up such that a fraction `percentile` of photons has
    travelled further than `cutoff_distance` after n steps, the path after n
    exponential steps being Erlang(n, sca_len)."""
    from scipy import stats
    n = int(np.ceil(cutoff_distance / sca_len))
    while stats.gamma.ppf(1.0 - percentile, n, scale=sca_len) <= cutoff_distance:
        n += 1
    return n


def resample_hits(hits: HitTable, replace: bool = False, rng=None) -> HitTable:
    """``resample_hits(hits, replace=false)`` (src/processing.jl:141-152): for
    each (module_id, pmt_id) a Poisson number of hits with mean the sum of
    their total_weight, drawn from them with probabilities proportional to
    the weights (without replacement unless `replace`)."""
    rng = rng if rng is not None else np.random.default_rng()
    mid = np.asarray(hits["module_id"]).astype(np.int64)
    pid = np.asarray(hits["pmt_id"]).astype(np.int64)
    w = np.asarray(hits["total_weight"], np.float64)
    keys = np.stack([mid, pid], axis=1)
    groups, inverse = np.unique(keys, axis=0, return_inverse=True)
    rows = []
    for g in range(len(groups)):
        idx = np.flatnonzero(inverse.reshape(-1) == g)
        wsum = w[idx].sum()
        k = int(rng.poisson(wsum))
        if k > len(idx) and not replace:
            raise ValueError(f"cannot draw {k} hits without replacement from {len(idx)}")
        rows.append(rng.choice(idx, size=k, replace=replace, p=w[idx] / wsum))
    take = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    out = HitTable()
    for key, v in hits.items():
        out[key] = np.asarray(v)[take]
    return out


def get_pmt_count(target) -> int:
    """PMTs of a module: 16 for a POM, 1 for a DOM or a homogeneous module, the
    layout's count for a multi-PMT module."""
    from .generic_multipmt import SphericalMultiPMTTarget
    from .generic_multipmt import get_pmt_count as multipmt_count
    from .pom import POM
    if isinstance(target, POM):
        return 16
    if isinstance(target, SphericalMultiPMTTarget):
        return multipmt_count(target)
    return 1


def add_pmt_noise(hits: list, targets, noise_rate: float = 1e4, time_window: float = 1e4,
                  rng=None, n_pmt: int | None = None) -> list:
    """``add_pmt_noise!(hits, targets; noise_rate=1E4, time_window=1E4)``
    (src/processing.jl:246-265): `hits` holds one array of hit times (ns) per
    (PMT, target), PMT fastest, n_pmt = get_pmt_count(first(targets)); each
    gets a Poisson number (mean noise_rate [Hz] * time_window [ns] * 1e-9) of
    times uniform on [-time_window / 2, time_window / 2], then is sorted.
    Returns `hits`."""
    rng = rng if rng is not None else np.random.default_rng()
    n_pmt = get_pmt_count(targets[0]) if n_pmt is None else int(n_pmt)
    mean = noise_rate * 1e-9 * time_window
    for tix in range(len(targets)):
        for pmt in range(n_pmt):
            i = pmt + n_pmt * tix
            k = int(rng.poisson(mean))
            if k > 0:
                noise = rng.uniform(-time_window / 2, time_window / 2, k)
                hits[i] = np.sort(np.concatenate([np.asarray(hits[i], np.float64), noise]))
    return hits
