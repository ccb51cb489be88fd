"""Optical modules and the detection step after propagation.

* ``POM``: the 16-PMT P-ONE optical module (src/pom.jl:63-112): a sphere of
  radius 0.3 m, PMTs of 75 mm diameter, PMT directions from
  ``make_pom_pmt_coordinates`` (src/pom.jl:114-142), the POMAcceptance tables
  (assets/pmt_acc.hd5) and the relative quantum efficiency (assets/PMTAcc.csv),
  both extracted into ``data/`` by ``data/extract_pom_tables.py``.
* ``make_hits_from_photons`` / ``calc_pe_weight`` (src/processing.jl:88-205):
  photon hits -> PMT hits, on the device (``pp_make_hits_from_photons``).

Deliberate differences: the random numbers come from a Philox stream keyed on
``seed`` and the hit's row (the reference uses Julia's global RNG); a
homogeneous module is detected with probability active_area / (4 pi r^2) as
PMT 1, the intent of check_pmt_hit(::HomogeneousTarget) (src/detection.jl:
70-84), whose signature the reference's make_hits_from_photons cannot call;
``calc_pe_weight`` applies the POM's relative QE table (the reference's
apply_qe(::POM) reads a field the model does not have, src/pom.jl:307).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib
from ._lib import check
from .targets import HomogeneousDetector, Spherical

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
POM_RADIUS = 0.3
POM_PMT_AREA = (75e-3 / 2) ** 2 * np.pi
POM_PMT_GROUP = np.array([1, 1, 1, 1, 2, 2, 2, 2, 1, 1, 1, 1, 2, 2, 2, 2], np.int32)  # pom.jl:161-163


@dataclass
class POM:
    """POM(position, module_id) (src/pom.jl:73-103) as a propagation target."""
    shape: Spherical
    module_id: int
    pmt_area: float = POM_PMT_AREA

    @classmethod
    def at(cls, position: Sequence[float], module_id: int) -> "POM":
        return cls(Spherical(list(position), POM_RADIUS), int(module_id))


def _sph_to_cart(theta, phi):
    return np.array([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)])


def _cart_to_sph(v):
    x, y, z = v
    return np.arccos(np.clip(z / np.linalg.norm(v), -1, 1)), np.arctan2(y, x)


def _rot_a_to_b(a, b):
    """Rotation matrix taking unit vector a onto b (Rodrigues)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    v = np.cross(a, b)
    c = float(np.dot(a, b))
    if np.linalg.norm(v) < 1e-15:
        return np.eye(3) if c > 0 else -np.eye(3)
    vx = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + vx + vx @ vx * (1.0 / (1.0 + c))


def make_pom_pmt_coordinates() -> np.ndarray:
    """(theta, phi) of the 16 PMTs, 2 x 16 (src/pom.jl:114-142): four rings
    at 90-25, 90-57.5, 90+25, 90+57.5 degrees, then turned by the rotation
    taking e_z onto e_x."""
    c = np.zeros((2, 16))
    c[0, 0:4] = np.deg2rad(90 - 25)
    c[1, 0:4] = np.arange(4) * np.pi / 2
    c[0, 4:8] = np.deg2rad(90 - 57.5)
    c[1, 4:8] = np.pi / 4 + np.arange(4) * np.pi / 2
    c[0, 8:12] = np.deg2rad(90 + 25)
    c[1, 8:12] = [np.pi / 2, 0, 3 * np.pi / 2, np.pi]
    c[0, 12:16] = np.deg2rad(90 + 57.5)
    c[1, 12:16] = [np.pi / 4, 7 / 4 * np.pi, 5 / 4 * np.pi, 3 / 4 * np.pi]
    R = _rot_a_to_b([0, 0, 1.0], [1.0, 0, 0])
    for i in range(16):
        c[:, i] = _cart_to_sph(R @ _sph_to_cart(c[0, i], c[1, i]))
    return c


def pom_pmt_directions(orientation=None) -> np.ndarray:
    """16 x 3 PMT unit vectors in the detector frame (orientation * the module
    frame; identity by default, as the reference's RotMatrix3(I))."""
    c = make_pom_pmt_coordinates()
    d = np.stack([_sph_to_cart(c[0, i], c[1, i]) for i in range(16)])
    if orientation is not None:
        d = d @ np.asarray(orientation, float).T
    return d


@dataclass
class POMTables:
    acc_wavelength: np.ndarray
    acc_group1: np.ndarray
    acc_group2: np.ndarray
    sigma_group1: float
    sigma_group2: float
    qe_wavelength: np.ndarray
    qe: np.ndarray


def load_pom_tables() -> POMTables:
    a = np.loadtxt(os.path.join(_DATA, "pom_pmt_acceptance.csv"), delimiter=",", skiprows=1)
    s = np.loadtxt(os.path.join(_DATA, "pom_pmt_sigma.csv"), delimiter=",", skiprows=1)
    q = np.loadtxt(os.path.join(_DATA, "pom_rel_qe.csv"), delimiter=",", skiprows=1)
    return POMTables(a[:, 0], a[:, 1], a[:, 2], float(s[0]), float(s[1]), q[:, 0], q[:, 1])


def pom_model(orientation=None, tables: POMTables | None = None) -> "_lib.pp_pom_model":
    t = tables or load_pom_tables()
    m = _lib.pp_pom_model()
    m.n_acc = len(t.acc_wavelength)
    m.n_qe = len(t.qe_wavelength)
    for name, arr in (("acc_wavelength", t.acc_wavelength), ("acc_group1", t.acc_group1),
                      ("acc_group2", t.acc_group2), ("qe_wavelength", t.qe_wavelength),
                      ("qe", t.qe)):
        dst = getattr(m, name)
        for i, v in enumerate(np.asarray(arr, np.float32)):
            dst[i] = float(v)
    m.sigma_group1 = t.sigma_group1
    m.sigma_group2 = t.sigma_group2
    d = pom_pmt_directions(orientation).astype(np.float32)
    for i in range(16):
        for k in range(3):
            m.pmt_dir[i][k] = float(d[i, k])
        m.pmt_group[i] = int(POM_PMT_GROUP[i])
    return m


def pmt_targets(targets) -> "ctypes.Array":
    """pp_pmt_target per propagation target (index i -> module_index i + 1)."""
    arr = (_lib.pp_pmt_target * max(1, len(targets)))()
    for i, t in enumerate(targets):
        p = np.asarray(t.shape.position, np.float32).reshape(3)
        arr[i].position[:] = (float(p[0]), float(p[1]), float(p[2]))
        arr[i].radius = float(np.float32(t.shape.radius))
        if isinstance(t, POM):
            arr[i].kind = _lib.PP_PMT_POM
            arr[i].active_area = float(t.pmt_area)
        elif isinstance(t, HomogeneousDetector):
            arr[i].kind = _lib.PP_PMT_HOMOGENEOUS
            arr[i].active_area = float(t.pmt_area)
        else:
            raise TypeError(f"target {i}: no detection model for {type(t).__name__}")
    return arr


def make_hits_device(d_records: int, n: int, targets, seed: int, d_pmt_id: int,
                     d_qe_weight: int = 0, orientation=None, stream: int = 0) -> None:
    """Device form: hit records in device memory -> PMT ids (and QE weights)."""
    lib = _lib.load()
    tg = pmt_targets(targets)
    pom = pom_model(orientation) if any(isinstance(t, POM) for t in targets) else None
    check(lib.pp_make_hits_from_photons(ctypes.c_void_p(d_records), int(n), tg, len(targets),
                                        ctypes.byref(pom) if pom is not None else None,
                                        int(seed), ctypes.c_void_p(d_pmt_id),
                                        ctypes.c_void_p(d_qe_weight or None),
                                        ctypes.c_void_p(stream)), "pp_make_hits_from_photons")


def records_from_table(table, targets) -> np.ndarray:
    """pp_hit_record rows (positions, wavelengths, 1-based module index) of a
    host hit table."""
    n = table.nrow
    rec = np.zeros(n, dtype=np.dtype(_lib.pp_hit_record))
    rec["position"] = np.asarray(table["position"], np.float32).reshape(n, 3)
    rec["wavelength"] = np.asarray(table["wavelength"], np.float32)
    index_of = {int(getattr(t, "module_id", i + 1)): i + 1 for i, t in enumerate(targets)}
    rec["module_index"] = np.array([index_of[int(m)] for m in table["module_id"]], np.int32) \
        if n else np.zeros(0, np.int32)
    return rec


def _targets_of(setup_or_targets):
    return getattr(setup_or_targets, "targets", setup_or_targets)


def make_hits_from_photons(table, setup_or_targets, target_orientation=None,
                           apply_wl_acc: bool = True, seed: int = 0, device: int = 0):
    """``make_hits_from_photons(df, setup_or_targets, target_orientation)``
    (src/processing.jl:88-139): the photons that a PMT detects, with a
    ``pmt_id`` column (1-based).  The POM's wavelength acceptance is part of
    its detection probability (its apply_wl_acceptance accepts all,
    src/pom.jl:165-174), so ``apply_wl_acc`` changes nothing here."""
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
                     orientation=target_orientation)
    ids = d_id.cpu().numpy()
    mask = ids > 0
    for k, v in table.items():
        out[k] = np.asarray(v)[mask]
    out["pmt_id"] = ids[mask]
    return out


def calc_pe_weight(table, setup_or_targets):
    """``calc_pe_weight!(photons, targets)`` (src/processing.jl:179-205): a
    ``qe_weight`` column (the POM's relative quantum efficiency at the
    wavelength, 0 outside the table; 1 for homogeneous modules) multiplied
    into ``total_weight``."""
    targets = _targets_of(setup_or_targets)
    t = load_pom_tables()
    is_pom = {int(getattr(x, "module_id", i + 1)): isinstance(x, POM) for i, x in enumerate(targets)}
    wl = np.asarray(table["wavelength"], np.float64)
    qe = np.interp(wl, t.qe_wavelength, t.qe, left=0.0, right=0.0)
    pom_rows = np.array([is_pom[int(m)] for m in table["module_id"]], bool) \
        if len(wl) else np.zeros(0, bool)
    qe = np.where(pom_rows, qe, 1.0)
    table["qe_weight"] = qe
    table["total_weight"] = np.asarray(table["total_weight"], np.float64) * qe
    return table
