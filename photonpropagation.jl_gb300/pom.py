"""The 16-PMT P-ONE optical module (mirrors src/pom.jl).

``POM``: a sphere of radius 0.3 m, PMTs of 75 mm diameter, PMT directions from
``make_pom_pmt_coordinates`` (src/pom.jl:114-142), the POMAcceptance tables
(assets/pmt_acc.hd5) and the relative quantum efficiency (assets/PMTAcc.csv),
both extracted into ``data/`` by ``data/extract_pom_tables.py``.  Detection
(check_pmt_hit for a POM, src/pom.jl:246-305) runs on the device; detection.py
drives it for every module kind.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib
from .targets import Spherical

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


POMAcceptance = POMTables  # the reference's name for the acceptance model (src/pom.jl:16-33)


class POMRelativeAcceptance:
    """The reference's relative-acceptance POM model (src/pom.jl:44-60), whose
    check_pmt_hit raises "Not Implemented" (src/pom.jl:190-197): detection
    with it raises here too."""

    def __init__(self, *args, **kwargs):
        raise NotImplementedError("POMRelativeAcceptance: check_pmt_hit is not implemented "
                                  "in the reference either")


def get_pom_pmt_group(pmt_ix: int) -> int:
    """Group (1 or 2) of the 1-based PMT index (src/pom.jl:160-162)."""
    return int(POM_PMT_GROUP[int(pmt_ix) - 1])

