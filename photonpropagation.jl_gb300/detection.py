"""The detection step after propagation (mirrors src/detection.jl and
make_hits_from_photons / calc_pe_weight!, src/processing.jl:88-205).

Photon hits -> PMT hits runs on the device (``pp_make_hits_from_photons_models``),
one thread per hit record, for every module kind:

* ``POM`` (pom.py): 16 PMTs, POMAcceptance;
* ``DOM`` (dom.py): angular polynomial, wavelength acceptance;
* ``SphericalMultiPMTTarget`` (generic_multipmt.py): projected-area hit
  probability, PMT chosen by a weighted sample;
* ``HomogeneousDetector``: active_area / (4 pi r^2), as PMT 1.

Deliberate differences: random numbers come from a Philox stream keyed on
``seed`` and the hit's row (the reference uses Julia's global RNG); a
homogeneous module is detected as PMT 1 with the probability that
check_pmt_hit(::HomogeneousTarget) (src/detection.jl:70-84) computes, whose
signature the reference's make_hits_from_photons cannot call; ``calc_pe_weight``
applies the POM's relative QE table (the reference's apply_qe(::POM) reads a
field the model does not have, src/pom.jl:307) and weight 1 for homogeneous
modules.  As in the reference, calc_pe_weight has no QE for a DOM
(apply_qe(::DOM) is not defined) and raises.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .dom import DOM, dom_model
from .generic_multipmt import InterpQuantumEff, SphericalMultiPMTTarget, multipmt_model
from .pom import POM, load_pom_tables, pom_model
from .targets import HomogeneousDetector


def check_pmt_hit_opening_angle(rel_hit_position, pmt_positions, opening_angle) -> int:
    """1-based index of the first PMT whose axis is within `opening_angle` of
    the (unit) relative hit position, 0 if none (src/detection.jl:33-44)."""
    rel = np.asarray(rel_hit_position, np.float64)
    for j, p in enumerate(np.asarray(pmt_positions, np.float64)):
        if np.arccos(np.clip(rel @ p, -1.0, 1.0)) < opening_angle:
            return j + 1
    return 0


def pmt_targets(targets) -> "ctypes.Array":
    """pp_pmt_target per propagation target (index i -> module_index i + 1)."""
    arr = (_lib.pp_pmt_target * max(1, len(targets)))()
    for i, t in enumerate(targets):
        p = np.asarray(t.shape.position, np.float32).reshape(3)
        arr[i].position[:] = (float(p[0]), float(p[1]), float(p[2]))
        arr[i].radius = float(np.float32(t.shape.radius))
        arr[i].active_area = float(getattr(t, "pmt_area", 0.0))
        if isinstance(t, POM):
            arr[i].kind = _lib.PP_PMT_POM
        elif isinstance(t, DOM):
            arr[i].kind = _lib.PP_PMT_DOM
        elif isinstance(t, SphericalMultiPMTTarget):
            arr[i].kind = _lib.PP_PMT_MULTIPMT
        elif isinstance(t, HomogeneousDetector):
            arr[i].kind = _lib.PP_PMT_HOMOGENEOUS
        else:
            raise TypeError(f"target {i}: no detection model for {type(t).__name__}")
    return arr


def detection_models(targets, orientation=None, apply_wl_acc: bool = True):
    """(pp_detection_models, the model structs it points to) for the kinds
    present in `targets`; keep the second item alive for the call."""
    keep = []
    models = _lib.pp_detection_models()
    if any(isinstance(t, POM) for t in targets):
        keep.append(pom_model(orientation))
        models.pom = ctypes.pointer(keep[-1])
    doms = [t for t in targets if isinstance(t, DOM)]
    if doms:
        keep.append(dom_model(doms[0].acceptance, orientation, apply_wl_acc))
        models.dom = ctypes.pointer(keep[-1])
    mps = [t for t in targets if isinstance(t, SphericalMultiPMTTarget)]
    if mps:
        keep.append(multipmt_model(mps, orientation))
        models.multipmt = ctypes.pointer(keep[-1])
    return models, keep


def make_hits_device(d_records: int, n: int, targets, seed: int, d_pmt_id: int,
                     d_qe_weight: int = 0, orientation=None, stream: int = 0,
                     apply_wl_acc: bool = True) -> None:
    """Device form: hit records in device memory -> PMT ids (and QE weights)."""
    lib = _lib.load()
    tg = pmt_targets(targets)
    models, keep = detection_models(targets, orientation, apply_wl_acc)
    check(lib.pp_make_hits_from_photons_models(
        ctypes.c_void_p(d_records), int(n), tg, len(targets), ctypes.byref(models), int(seed),
        ctypes.c_void_p(d_pmt_id), ctypes.c_void_p(d_qe_weight or None),
        ctypes.c_void_p(stream)), "pp_make_hits_from_photons_models")
    del keep


def records_from_table(table, targets) -> np.ndarray:
    """pp_hit_record rows (positions, directions, wavelengths, 1-based module
    index) of a host hit table."""
    n = table.nrow
    rec = np.zeros(n, dtype=np.dtype(_lib.pp_hit_record))
    rec["position"] = np.asarray(table["position"], np.float32).reshape(n, 3)
    if "direction" in table:
        rec["direction"] = np.asarray(table["direction"], np.float32).reshape(n, 3)
    rec["wavelength"] = np.asarray(table["wavelength"], np.float32)
    index_of = {int(getattr(t, "module_id", i + 1)): i + 1 for i, t in enumerate(targets)}
    rec["module_index"] = np.array([index_of[int(m)] for m in table["module_id"]], np.int32) \
        if n else np.zeros(0, np.int32)
    return rec


def _targets_of(setup_or_targets):
    return getattr(setup_or_targets, "targets", setup_or_targets)


def make_hits_from_photons(table, setup_or_targets, target_orientation=None,
                           apply_wl_acc: bool = True, seed: int = 0, device: int = 0):
    """``make_hits_from_photons(df, setup_or_targets, target_orientation,
    apply_wl_acc)`` (src/processing.jl:88-139): the photons that a PMT detects,
    with a ``pmt_id`` column (1-based).  ``apply_wl_acc`` matters for DOMs
    only: the POM's and the multi-PMT module's apply_wl_acceptance accept all
    (src/pom.jl:165-174, src/detection.jl:141-146)."""
    import torch
    from .processing import HitTable
    targets = _targets_of(setup_or_targets)
    rec = records_from_table(table, targets)
    n = len(rec)
    out = HitTable()
    if n == 0:
        for k, v in table.items():
            out[k] = v
        out["pmt_id"] = np.zeros(0, np.int32)
        return out
    d_rec = torch.from_numpy(rec.view(np.uint8)).to(f"cuda:{device}")
    d_id = torch.empty(n, dtype=torch.int32, device=f"cuda:{device}")
    make_hits_device(d_rec.data_ptr(), n, targets, seed, d_id.data_ptr(),
                     orientation=target_orientation, apply_wl_acc=apply_wl_acc)
    ids = d_id.cpu().numpy()
    mask = ids > 0
    for k, v in table.items():
        out[k] = np.asarray(v)[mask]
    out["pmt_id"] = ids[mask]
    return out


def apply_qe(wl, target) -> np.ndarray:
    """QE weight of hits on `target` (apply_qe, src/detection.jl:188)."""
    wl = np.asarray(wl, np.float64)
    if isinstance(target, POM):
        t = load_pom_tables()
        return np.interp(wl, t.qe_wavelength, t.qe, left=0.0, right=0.0)
    if isinstance(target, SphericalMultiPMTTarget):
        if target.wl_acceptance is None:
            raise TypeError("apply_qe: the multi-PMT module has no wl_acceptance")
        return target.wl_acceptance(wl)
    if isinstance(target, HomogeneousDetector):
        return np.ones_like(wl)
    raise NotImplementedError(f"apply_qe not implemented for type {type(target).__name__}")


def calc_pe_weight(table, setup_or_targets):
    """``calc_pe_weight!(photons, targets)`` (src/processing.jl:179-205): a
    ``qe_weight`` column multiplied into ``total_weight``."""
    targets = _targets_of(setup_or_targets)
    by_id = {int(getattr(x, "module_id", i + 1)): x for i, x in enumerate(targets)}
    wl = np.asarray(table["wavelength"], np.float64)
    mid = np.asarray(table["module_id"]).astype(np.int64) if len(wl) else np.zeros(0, np.int64)
    qe = np.zeros(len(wl))
    for m in np.unique(mid):
        rows = mid == m
        qe[rows] = apply_qe(wl[rows], by_id[int(m)])
    table["qe_weight"] = qe
    table["total_weight"] = np.asarray(table["total_weight"], np.float64) * qe
    return table


def check_pmt_hit(hit_positions, hit_directions, hit_wavelengths, target, orientation=None,
                  seed: int = 0, device: int = 0) -> np.ndarray:
    """``check_pmt_hit(positions, directions, wavelengths, target, orientation)``
    (src/detection.jl:51-131, src/pom.jl:246-305, src/dom.jl:96-116): the 1-based
    PMT of each photon on `target` (0 = not detected), on the device.  For a
    DOM only the angular acceptance, as the reference (its wavelength test is
    ``apply_wl_acceptance``)."""
    import torch
    pos = np.asarray(hit_positions, np.float32).reshape(-1, 3)
    n = len(pos)
    if n == 0:
        return np.zeros(0, np.int32)
    rec = np.zeros(n, dtype=np.dtype(_lib.pp_hit_record))
    rec["position"] = pos
    rec["direction"] = np.asarray(hit_directions, np.float32).reshape(-1, 3)
    rec["wavelength"] = np.asarray(hit_wavelengths, np.float32).reshape(-1) \
        if len(np.atleast_1d(hit_wavelengths)) else 0.0
    rec["module_index"] = 1
    d_rec = torch.from_numpy(rec.view(np.uint8)).to(f"cuda:{device}")
    d_id = torch.empty(n, dtype=torch.int32, device=f"cuda:{device}")
    make_hits_device(d_rec.data_ptr(), n, [target], seed, d_id.data_ptr(),
                     orientation=orientation, apply_wl_acc=False)
    return d_id.cpu().numpy()


def apply_wl_acceptance(hit_positions, hit_directions, hit_wavelengths, target,
                        orientation=None, rng=None) -> np.ndarray:
    """``apply_wl_acceptance`` (src/dom.jl:122-134, src/pom.jl:165-174,
    src/detection.jl:141-146): a DOM keeps a photon when u < wl_acc(wavelength);
    POMs and multi-PMT modules keep all."""
    wl = np.asarray(hit_wavelengths, np.float64).reshape(-1)
    if isinstance(target, DOM):
        rng = rng if rng is not None else np.random.default_rng()
        return rng.uniform(size=len(wl)) < target.acceptance.wavelength(wl)
    if isinstance(target, (POM, SphericalMultiPMTTarget)):
        return np.ones(len(np.asarray(hit_positions).reshape(-1, 3)), bool)
    raise NotImplementedError(f"apply_wl_acceptance not implemented for {type(target).__name__}")

