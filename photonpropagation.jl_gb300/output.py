"""Event output tables (mirrors src/output.jl).

Hit lists (one array of hit times per (PMT, module), PMT fastest, as
``add_pmt_noise`` takes them) to and from hit tables, module and source
tables, and ``save_event``.  The reference writes events into HDF5 groups
``/hits/<event_id>`` and ``/sources/<event_id>/<source type>``; h5py is not
available here, so the same layout is kept as directories of ``.npz`` files
(``read_event`` reads one back).
"""
from __future__ import annotations

import os

import numpy as np

from .processing import HitTable, get_pmt_count


def hit_list_to_dataframe(hit_list, targets, target_mask=None) -> HitTable:
    """``hit_list_to_dataframe(hit_list, targets, target_mask)`` (src/output.jl:20-33):
    a table of (time, pmt_id, module_id), one row per hit."""
    sel = [t for t, keep in zip(targets, target_mask if target_mask is not None
                                else [True] * len(targets)) if keep]
    n_pmt = get_pmt_count(sel[0]) if sel else 0
    times, pmts, mods = [], [], []
    for i, hits in enumerate(hit_list):
        target = sel[i // n_pmt]
        h = np.asarray(hits, np.float64)
        times.append(h)
        pmts.append(np.full(len(h), i % n_pmt + 1, np.int64))
        mods.append(np.full(len(h), int(target.module_id), np.int64))
    cat = lambda xs, dt: np.concatenate(xs) if xs else np.zeros(0, dt)  # noqa: E731
    return HitTable(time=cat(times, np.float64), pmt_id=cat(pmts, np.int64),
                    module_id=cat(mods, np.int64))


def dataframe_to_hit_list(hits, targets) -> list:
    """``dataframe_to_hit_list(hits, targets)`` (src/output.jl:36-48): the hit
    times of every (PMT, module), PMT fastest."""
    n_pmt = get_pmt_count(targets[0])
    t = np.asarray(hits["time"], np.float64)
    m = np.asarray(hits["module_id"]).astype(np.int64)
    p = np.asarray(hits["pmt_id"]).astype(np.int64)
    return [t[(m == int(target.module_id)) & (p == pmt)] for target in targets
            for pmt in range(1, n_pmt + 1)]


def targets_to_dataframe(targets) -> HitTable:
    """``targets_to_dataframe(targets)`` (src/output.jl:51-71): one row per
    PMT with the module position and the PMT's (theta, phi)."""
    from .pom import make_pom_pmt_coordinates
    cols = {k: [] for k in ("module_id", "pmt_id", "module_x", "module_y", "module_z",
                            "pmt_theta", "pmt_phi")}
    for t in targets:
        coords = getattr(t, "pmt_coordinates", None)
        if coords is None:
            coords = make_pom_pmt_coordinates()
        coords = np.asarray(coords, np.float64)
        for j in range(coords.shape[1]):
            cols["module_id"].append(int(t.module_id))
            cols["pmt_id"].append(j + 1)
            for a, k in zip(t.shape.position, ("module_x", "module_y", "module_z")):
                cols[k].append(float(a))
            cols["pmt_theta"].append(coords[0, j])
            cols["pmt_phi"].append(coords[1, j])
    return HitTable({k: np.asarray(v) for k, v in cols.items()})


def event_info_to_dataframe(particle) -> HitTable:
    """``event_info_to_dataframe(particle)`` (src/output.jl:73-87): one row."""
    p, d = particle.position, particle.direction
    return HitTable({k: np.array([v], np.float64) for k, v in (
        ("x", p[0]), ("y", p[1]), ("z", p[2]), ("dir_x", d[0]), ("dir_y", d[1]), ("dir_z", d[2]),
        ("time", particle.time), ("energy", particle.energy), ("length", particle.length))})


def source_to_namedtuple(source) -> dict:
    """``source_to_namedtuple`` (src/output.jl:91-103)."""
    return dict(location_x=source.position[0], location_y=source.position[1],
                location_z=source.position[2], direction_x=source.direction[0],
                direction_y=source.direction[1], direction_z=source.direction[2],
                time=source.time, n_photons=int(source.photons))


def save_event(path: str, event_record: dict) -> None:
    """``save_event(path, event_record)`` (src/output.jl:113-135): the event's
    hits (time, module_id, pmt_id) under ``hits/<event_id>.npz`` and its
    sources, grouped by type, under ``sources/<event_id>/<type>.npz``."""
    eid = str(event_record["event_id"])
    hits = event_record["hits"]
    os.makedirs(os.path.join(path, "hits"), exist_ok=True)
    np.savez(os.path.join(path, "hits", eid + ".npz"),
             **{k: np.asarray(hits[k]) for k in ("time", "module_id", "pmt_id")})
    by_type = {}
    for s in event_record.get("sources", []):
        by_type.setdefault(type(s).__name__, []).append(source_to_namedtuple(s))
    sdir = os.path.join(path, "sources", eid)
    os.makedirs(sdir, exist_ok=True)
    for name, rows in by_type.items():
        np.savez(os.path.join(sdir, name + ".npz"),
                 **{k: np.array([r[k] for r in rows]) for k in rows[0]})


def read_event(path: str, event_id) -> dict:
    """The tables ``save_event`` wrote for `event_id`."""
    eid = str(event_id)
    with np.load(os.path.join(path, "hits", eid + ".npz")) as f:
        hits = HitTable({k: f[k] for k in f.files})
    sources = {}
    sdir = os.path.join(path, "sources", eid)
    for fn in sorted(os.listdir(sdir)) if os.path.isdir(sdir) else []:
        with np.load(os.path.join(sdir, fn)) as f:
            sources[fn[:-4]] = {k: f[k] for k in f.files}
    return dict(event_id=event_id, hits=hits, sources=sources)
