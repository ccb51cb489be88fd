"""propagate_photons and its helpers (mirrors src/processing.jl:32-75 and
src/photon_prop_cuda.jl:878-959)."""
from __future__ import annotations

import numpy as np

from . import _lib
from .context import Context, device_memory
from .sources import to_records
from . import targets as _targets
from .targets import module_ids

_CONTEXTS: dict = {}


class PhotonPropOOMException(Exception):
    """The hit buffer was too small (src/photon_prop_cuda.jl:40, :937-939)."""


class HitTable(dict):
    """Column table of hits (the reference returns a DataFrame with these
    columns; numpy arrays keyed by column name here)."""

    @property
    def nrow(self) -> int:
        return int(self["wavelength"].shape[0]) if "wavelength" in self else 0


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
    key = (id(ctx), id(setup.medium), id(setup.spec_dist), _targets.identity(setup.targets),
           setup.needs_track_smear())
    if getattr(setup, "_uploaded_key", None) != key:
        setup.upload(ctx)
        setup._uploaded_key = key


def _run(setup, hit_buffers: HitBuffers, n_steps: int):
    ctx = get_context(hit_buffers.device)
    _ensure_uploaded(setup, ctx)
    recs = to_records(setup.sources)
    rc, n_hits, n_ph_sim = ctx.propagate(recs, len(setup.sources), setup.seed, n_steps,
                                         setup.photon_scaling, hit_buffers.capacity)
    if rc == _lib.PP_ERR_OVERFLOW:
        raise PhotonPropOOMException(
            f"{n_hits} hits exceed the hit buffer capacity {hit_buffers.capacity}")
    return ctx.fetch_hits(n_hits), n_ph_sim


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
