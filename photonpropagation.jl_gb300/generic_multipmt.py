"""The generic spherical multi-PMT module (mirrors src/generic_multipmt.jl and
the SphericalMultiPMTTarget methods of src/detection.jl:90-131).

``make_generic_multipmt_om(position, radius, module_id)`` places 20 PMTs of
76.2 mm diameter at the (theta, phi) of ``make_generic_multipmt_positions``
with the R6091 quantum efficiency (QE / 100, ``data/multipmt_qe.csv``).
The PMT axes are ``sph_to_cart(theta, phi)`` turned by the module orientation
(the unexported ``get_pmt_positions`` of NeutrinoTelescopeBase 1.0.0-DEV,
restated: the package is not available to pin it against).

Detection runs on the device in ``pp_make_hits_from_photons_models``.
"""
from __future__ import annotations

import os
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib
from .targets import Spherical

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

# (theta; phi) of the 20 PMTs, src/generic_multipmt.jl:27-31
_GENERIC_PMT_COORDINATES = np.array([
    [2.25125, 0.634634, 1.14901, 1.65559, 0.899014, 1.69387, 0.186803, 2.51845, 0.745349,
     1.04614, 2.16353, 0.962081, 1.4594, 2.00863, 1.74027, 1.47242, 2.38773, 2.94739, 2.08877,
     1.40132],
    [6.01403, 5.77419, 4.92832, 2.4311, 4.00995, 4.24677, 2.99576, 4.22343, 0.843871, 3.01157,
     1.74808, 1.98313, 5.76502, 5.08536, 3.43438, 1.29802, 2.87137, 0.808321, 0.726752,
     0.292785]])


def fibonacci_sphere(n: int) -> np.ndarray:
    """n points on the unit sphere by the golden-angle spiral (src/generic_multipmt.jl:3-22)."""
    i = np.arange(n, dtype=np.float64)
    y = 1.0 - i / (n - 1) * 2.0
    radius = np.sqrt(1.0 - y * y)
    theta = np.pi * (3.0 - np.sqrt(5.0)) * i
    return np.stack([np.cos(theta) * radius, y, np.sin(theta) * radius], axis=1)


def make_generic_multipmt_positions() -> np.ndarray:
    """2 x 20 (theta, phi) of the PMTs."""
    return _GENERIC_PMT_COORDINATES.copy()


def load_multipmt_qe():
    q = np.loadtxt(os.path.join(_DATA, "multipmt_qe.csv"), delimiter=",", skiprows=1)
    return q[:, 0], q[:, 1]


class InterpQuantumEff:
    """InterpQuantumEff (src/detection.jl:163-186): linear interpolation of a
    QE table, 0 outside it.  ``from_csv(path, relative)`` reads the reference's
    CSV format: QE / 100, or the rel_acceptance column when ``relative``."""

    def __init__(self, wavelength, qe):
        self.wavelength = np.asarray(wavelength, np.float64)
        self.qe = np.asarray(qe, np.float64)

    @classmethod
    def from_csv(cls, path, relative: bool = False):
        import csv
        with open(path, newline="") as f:
            rows = list(csv.DictReader(f))
        wl = [float(r["wavelength"]) for r in rows]
        y = [float(r["rel_acceptance"]) if relative else float(r["QE"]) / 100.0 for r in rows]
        return cls(wl, y)

    def __call__(self, wl):
        return np.interp(np.asarray(wl, np.float64), self.wavelength, self.qe, left=0.0, right=0.0)


@dataclass
class SphericalMultiPMTTarget:
    """SphericalMultiPMTTarget(shape, pmt_area, pmt_coordinates, wl_acceptance,
    module_id) as NeutrinoTelescopeBase defines it: pmt_coordinates 2 x n_pmt
    (theta; phi), wl_acceptance an InterpQuantumEff (or None, as in the
    reference's example; calc_pe_weight then has no QE to apply)."""
    shape: Spherical
    pmt_area: float
    pmt_coordinates: np.ndarray
    wl_acceptance: "InterpQuantumEff | None"
    module_id: int


def make_generic_multipmt_om(position: Sequence[float], radius: float, module_id: int,
                             pmt_diameter: float = 0.0762) -> SphericalMultiPMTTarget:
    """make_generic_multipmt_om (src/generic_multipmt.jl:35-52)."""
    return SphericalMultiPMTTarget(Spherical(list(position), float(radius)),
                                   (pmt_diameter / 2) ** 2 * np.pi,
                                   make_generic_multipmt_positions(),
                                   InterpQuantumEff(*load_multipmt_qe()), int(module_id))


def get_pmt_count(target: SphericalMultiPMTTarget) -> int:
    return int(np.asarray(target.pmt_coordinates).shape[1])


def get_pmt_positions(target: SphericalMultiPMTTarget, orientation=None) -> np.ndarray:
    """n_pmt x 3 unit axes: orientation * sph_to_cart(theta, phi)."""
    th, ph = np.asarray(target.pmt_coordinates, np.float64)
    d = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
    if orientation is not None:
        d = d @ np.asarray(orientation, np.float64).T
    return d


def _qe_knots(t: SphericalMultiPMTTarget):
    """QE knots for the device; a target without wl_acceptance gets weight 1."""
    if t.wl_acceptance is None:
        return np.array([0.0, 1e4]), np.array([1.0, 1.0])
    return t.wl_acceptance.wavelength, t.wl_acceptance.qe


def _layout_key(t: SphericalMultiPMTTarget):
    wl, qe = _qe_knots(t)
    return (float(t.pmt_area), np.asarray(t.pmt_coordinates, np.float64).tobytes(),
            np.asarray(wl, np.float64).tobytes(), np.asarray(qe, np.float64).tobytes())


def multipmt_model(targets: Sequence[SphericalMultiPMTTarget],
                   orientation=None) -> "_lib.pp_multipmt_model":
    """pp_multipmt_model shared by the multi-PMT modules of one detection call
    (they must share PMT layout, area and QE table)."""
    t0 = targets[0]
    key = _layout_key(t0)
    if any(_layout_key(t) != key for t in targets[1:]):
        raise ValueError("multi-PMT modules of one call must share PMT layout, area and QE")
    n = get_pmt_count(t0)
    if not 1 <= n <= _lib.PP_MULTIPMT_MAX_PMTS:
        raise ValueError(f"{n} PMTs exceed the device limit {_lib.PP_MULTIPMT_MAX_PMTS}")
    qwl, qv = _qe_knots(t0)
    if not 2 <= len(qwl) <= _lib.PP_POM_MAX_KNOTS:
        raise ValueError("multi-PMT QE table needs 2..128 knots")
    m = _lib.pp_multipmt_model()
    m.n_pmt = n
    m.n_qe = len(qwl)
    m.pmt_area = float(t0.pmt_area)
    dm = get_pmt_positions(t0).astype(np.float32)
    do = get_pmt_positions(t0, orientation).astype(np.float32)
    for i in range(n):
        m.pmt_dir_module[i][:] = [float(v) for v in dm[i]]
        m.pmt_dir[i][:] = [float(v) for v in do[i]]
    for i, (x, y) in enumerate(zip(np.asarray(qwl, np.float32), np.asarray(qv, np.float32))):
        m.qe_wavelength[i] = float(x)
        m.qe[i] = float(y)
    return m
