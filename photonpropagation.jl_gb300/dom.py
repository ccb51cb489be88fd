"""The single-PMT DOM (mirrors src/dom.jl).

``DOM(position, module_id)`` is a sphere of radius 0.16510 m with a 12-inch PMT
(area pi * 0.1524^2) and a ``DOMAcceptance``: an angular acceptance polynomial
in the cosine of the photon direction's zenith in the module frame, with its
maximum ``polymax``, and a wavelength acceptance (effective area over the
DOM's cross-section).  The tables come from the reference's assets through
``data/extract_detection_tables.py``.

Detection (check_pmt_hit and apply_wl_acceptance for a DOM, src/dom.jl:96-134)
runs on the device in ``pp_make_hits_from_photons_models``.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib
from .targets import Spherical

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DOM_RADIUS = 0.16510
DOM_PMT_AREA = (0.3048 / 2) ** 2 * np.pi


@dataclass
class DOMAcceptance:
    """DOMAcceptance(poly_ang, polymax, int_wl) (src/dom.jl:8-26): polynomial
    coefficients in ascending powers of cos(zenith), its maximum, and the
    wavelength acceptance knots (0 outside them)."""
    poly: np.ndarray
    polymax: float
    wl: np.ndarray
    wl_acc: np.ndarray

    def angular(self, coszenith):
        """poly_ang(cos zenith), FP64 (Horner)."""
        x = np.asarray(coszenith, np.float64)
        out = np.zeros_like(x)
        for c in self.poly[::-1]:
            out = out * x + c
        return out

    def wavelength(self, wl):
        """int_wl(wavelength): linear, 0 outside the table."""
        return np.interp(np.asarray(wl, np.float64), self.wl, self.wl_acc, left=0.0, right=0.0)


def load_dom_acceptance() -> DOMAcceptance:
    v = np.loadtxt(os.path.join(_DATA, "dom_angular_acceptance.csv"), comments="#")
    w = np.loadtxt(os.path.join(_DATA, "dom_wl_acceptance.csv"), delimiter=",", skiprows=1)
    return DOMAcceptance(v[1:], float(v[0]), w[:, 0], w[:, 1])


@dataclass
class DOM:
    """DOM(position, module_id) (src/dom.jl:29-66) as a propagation target."""
    shape: Spherical
    module_id: int
    pmt_area: float = DOM_PMT_AREA
    acceptance: DOMAcceptance = field(default_factory=load_dom_acceptance, repr=False)

    @classmethod
    def at(cls, position: Sequence[float], module_id: int) -> "DOM":
        return cls(Spherical(list(position), DOM_RADIUS), int(module_id))


def get_pmt_count(_dom=None) -> int:
    return 1


def dom_model(acceptance: DOMAcceptance | None = None, orientation=None,
              apply_wl_acc: bool = True) -> "_lib.pp_dom_model":
    """pp_dom_model: cos zenith = (inv(orientation) * direction)[3] = the third
    column of the orientation dotted with the direction."""
    a = acceptance or load_dom_acceptance()
    if not 1 <= len(a.poly) <= _lib.PP_DOM_MAX_POLY:
        raise ValueError(f"DOM polynomial of degree {len(a.poly) - 1} exceeds the device limit")
    if not 2 <= len(a.wl) <= _lib.PP_POM_MAX_KNOTS:
        raise ValueError("DOM wavelength table needs 2..128 knots")
    m = _lib.pp_dom_model()
    m.n_poly = len(a.poly)
    m.n_wl = len(a.wl)
    for i, c in enumerate(np.asarray(a.poly, np.float32)):
        m.poly[i] = float(c)
    m.polymax = float(a.polymax)
    R = np.eye(3) if orientation is None else np.asarray(orientation, np.float64)
    m.zenith_axis[:] = [float(v) for v in R[:, 2].astype(np.float32)]
    for i, (x, y) in enumerate(zip(np.asarray(a.wl, np.float32), np.asarray(a.wl_acc, np.float32))):
        m.wl[i] = float(x)
        m.wl_acc[i] = float(y)
    m.apply_wl_acceptance = 1 if apply_wl_acc else 0
    return m
