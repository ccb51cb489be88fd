"""Synthetic workloads with the shapes of the benchmark configurations.

C0  README example: isotropic point at the origin, 450 nm, one sphere
    (r = 0.3 m) at (0, 0, 10) m.
C1  400 modules (r = 0.2159 m) on 20 vertical strings, string x/y uniform in
    a 500 m x 500 m square, modules every 25 m from z = -250 to +225 m; one
    isotropic point uniform inside the detector hull; Frank-Tamm spectrum on
    300-800 nm.
C2  The C1 detector with 256 emitters uniform in a 1 km cube centred on it,
    directions uniform on the sphere, half point-isotropic and half extended
    Cherenkov cascades (a = 2.0, b = 0.63, lrad = 0.36 m), photon counts
    log-uniform on [1e4, 1e7].
All inputs are seeded and generated here; no external data is used.
"""
from __future__ import annotations

import numpy as np

from .medium import CascadiaMediumProperties
from .propsetup import PhotonPropSetup
from .sources import (ExtendedCherenkovEmitter, LongitudinalParameterisation,
                      PointlikeIsotropicEmitter)
from .spectrum import make_cherenkov_spectrum, make_monochromatic_spectrum
from .targets import HomogeneousDetector, Spherical

PMT_AREA = 16 * np.pi * 0.0762 ** 2


def c0_setup(photons: int = 100_000, seed: int = 1, medium=None) -> PhotonPropSetup:
    medium = medium or CascadiaMediumProperties(0.95, 0.2, 1.0, 1.0)
    target = HomogeneousDetector(Spherical([0.0, 0.0, 10.0], 0.3), PMT_AREA, 1)
    src = PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, photons)
    return PhotonPropSetup([src], [target], medium, make_monochromatic_spectrum(450.0), seed)


def detector_400(rng_seed: int = 1234, radius: float = 0.2159):
    """The 400-module detector; returns (targets, string_xy)."""
    rng = np.random.default_rng(rng_seed)
    xy = rng.uniform(-250.0, 250.0, size=(20, 2))
    targets = []
    mid = 1
    for s in range(20):
        for k in range(20):
            z = -250.0 + 25.0 * k
            targets.append(HomogeneousDetector(Spherical([xy[s, 0], xy[s, 1], z], radius),
                                               PMT_AREA, mid))
            mid += 1
    return targets, xy


def point_in_hull(xy: np.ndarray, rng) -> list:
    """Uniform point inside the detector hull: the convex hull of the strings in
    x/y times the z span of the modules."""
    from scipy.spatial import Delaunay
    tri = Delaunay(xy)
    lo, hi = xy.min(axis=0), xy.max(axis=0)
    while True:
        p = rng.uniform(lo, hi)
        if tri.find_simplex(p) >= 0:
            return [float(p[0]), float(p[1]), float(rng.uniform(-250.0, 225.0))]


def c1_setup(photons: int = 100_000_000, seed: int = 1, rng_seed: int = 1234) -> PhotonPropSetup:
    medium = CascadiaMediumProperties(0.95, 0.2, 1.0, 1.0)
    targets, xy = detector_400(rng_seed)
    pos = point_in_hull(xy, np.random.default_rng(rng_seed + 1000 * seed))
    src = PointlikeIsotropicEmitter(pos, 0.0, photons)
    spec = make_cherenkov_spectrum((300.0, 800.0), medium)
    return PhotonPropSetup([src], targets, medium, spec, seed)


def unit_vectors(rng, n: int) -> np.ndarray:
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def c2_sources(n: int = 256, rng_seed: int = 4321, lo: float = 1e4, hi: float = 1e7,
               scale: float = 1.0):
    """Half point-isotropic, half extended-Cherenkov emitters in a 1 km cube;
    photon counts log-uniform on [lo, hi] (times `scale`)."""
    rng = np.random.default_rng(rng_seed)
    pos = rng.uniform(-500.0, 500.0, size=(n, 3))
    dirs = unit_vectors(rng, n)
    counts = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n)) * scale
    lp = LongitudinalParameterisation(2.0, 0.63, 0.36)
    out = []
    for i in range(n):
        c = max(1, int(round(counts[i])))
        if i % 2 == 0:
            out.append(PointlikeIsotropicEmitter(pos[i], 0.0, c))
        else:
            out.append(ExtendedCherenkovEmitter(pos[i], dirs[i], 0.0, c, lp))
    return out


def c2_setup(n_sources: int = 256, seed: int = 1, rng_seed: int = 1234, scale: float = 1.0):
    medium = CascadiaMediumProperties(0.95, 0.2, 1.0, 1.0)
    targets, _ = detector_400(rng_seed)
    spec = make_cherenkov_spectrum((300.0, 800.0), medium)
    return PhotonPropSetup(c2_sources(n_sources, scale=scale), targets, medium, spec, seed)
