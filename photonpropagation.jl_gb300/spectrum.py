"""Wavelength spectra (mirrors PhotonPropagation.jl src/spectrum.jl).

``make_cherenkov_spectrum`` builds the cumulative distribution of the
Frank-Tamm spectrum at 1 nm steps with 25-point Gauss-Legendre quadrature
(make_spectral_dist, src/spectrum.jl:41-62) and inverts it by linear
interpolation; ``device_knots`` evaluates that inverse CDF at
``spectrum_interp_steps`` equally spaced probabilities, the table the device
samples like the reference's 1-D texture (make_cuda_spectral_dist,
src/spectrum.jl:75-83).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Tuple

import numpy as np

FINE_STRUCTURE = 7.2973525693e-3


def frank_tamm(wl, ref_index):
    """Frank-Tamm photon yield per unit length and wavelength (wl in nm, beta=1)."""
    wl = np.asarray(wl, np.float64)
    n = np.asarray(ref_index, np.float64)
    return 2.0 * np.pi * FINE_STRUCTURE / wl ** 2 * (1.0 - 1.0 / n ** 2)


_GL_CACHE = {}


def integrate_gauss_quad(f: Callable, a: float, b: float, order: int = 25) -> float:
    """Gauss-Legendre quadrature of f on [a, b] (integrate_gauss_quad, PhysicsTools)."""
    if order not in _GL_CACHE:
        _GL_CACHE[order] = np.polynomial.legendre.leggauss(order)
    x, w = _GL_CACHE[order]
    half = 0.5 * (b - a)
    mid = 0.5 * (b + a)
    return float(half * np.sum(w * f(mid + half * x)))


class SpectralDist:
    pass


@dataclass
class Monochromatic(SpectralDist):
    """Monochromatic spectrum (src/spectrum.jl:66-72)."""
    wavelength: float


@dataclass
class InterpolatedSpectralDist(SpectralDist):
    """Inverse CDF as a piecewise-linear map from CDF value to wavelength."""
    cdf: np.ndarray          # increasing CDF values at the knots
    wavelengths: np.ndarray  # knot wavelengths (nm)
    normalization: float

    def inverse_cdf(self, u):
        u = np.asarray(u, np.float64)
        out = np.interp(u, self.cdf, self.wavelengths)
        # extrapolation_bc = 0 outside the knot range
        return np.where((u < self.cdf[0]) | (u > self.cdf[-1]), 0.0, out)

    def device_knots(self, interp_steps: int = 600) -> np.ndarray:
        """The table the device samples: inverse CDF at range(0, 1, interp_steps)."""
        return np.asarray(self.inverse_cdf(np.linspace(0.0, 1.0, interp_steps)), np.float32)


@dataclass
class Spectrum:
    """Spectral distribution + the spectrum function + its wavelength range."""
    spectral_dist: SpectralDist
    spectrum: Callable
    wl_range: Tuple[float, float]


def make_spectral_dist(spect_func: Callable, wl_range, step_size: float = 1.0):
    """CDF at wl_range[0]:step:wl_range[1] by Gauss quadrature; returns the inverse
    CDF (src/spectrum.jl:41-62)."""
    lo, hi = float(wl_range[0]), float(wl_range[1])
    wl_steps = np.arange(lo, hi + 0.5 * step_size, step_size, dtype=np.float64)
    wl_steps = wl_steps[wl_steps <= hi + 1e-9]
    full_norm = integrate_gauss_quad(spect_func, lo, hi, 25)
    norms = np.zeros_like(wl_steps)
    for i in range(1, len(wl_steps)):
        norms[i] = integrate_gauss_quad(spect_func, lo, wl_steps[i], 25) / full_norm
    # deduplicate_knots!(move_knots=true): nudge repeated values upward
    for i in range(1, len(norms)):
        if norms[i] <= norms[i - 1]:
            norms[i] = np.nextafter(norms[i - 1], np.inf)
    order = np.argsort(norms, kind="stable")
    return InterpolatedSpectralDist(norms[order], wl_steps[order], full_norm)


def make_cherenkov_spectrum(wl_range, medium) -> Spectrum:
    """Frank-Tamm spectrum in `medium` (src/spectrum.jl:91-95)."""
    def sfunc(wl):
        return frank_tamm(wl, medium.phase_refractive_index(wl)) * 1e9
    return Spectrum(make_spectral_dist(sfunc, wl_range), sfunc,
                    (float(wl_range[0]), float(wl_range[1])))


def make_cuda_spectral_dist(spec: SpectralDist, wl_range=None, interp_steps: int = 30):
    """``make_cuda_spectral_dist(spec, wl_range, interp_steps)`` (src/spectrum.jl:75-83):
    the inverse CDF sampled at `interp_steps` points of [0, 1] that the device
    interpolates (PhotonPropSetup uses 600); a Monochromatic passes through."""
    if isinstance(spec, Monochromatic):
        return spec
    return spec.device_knots(interp_steps)


def make_biased_cherenkov_spectrum(bias_function: Callable, wl_range, medium) -> Spectrum:
    """Frank-Tamm spectrum times `bias_function(wl)` (e.g. a module's wavelength
    acceptance), its CDF tabulated every 0.5 nm (src/spectrum.jl:97-101)."""
    def sfunc(wl):
        return frank_tamm(wl, medium.phase_refractive_index(wl)) * bias_function(wl) * 1e9
    return Spectrum(make_spectral_dist(sfunc, wl_range, 0.5), sfunc,
                    (float(wl_range[0]), float(wl_range[1])))


def make_monochromatic_spectrum(wl: float) -> Spectrum:
    """src/spectrum.jl:103-105"""
    return Spectrum(Monochromatic(float(wl)), lambda w: np.where(np.asarray(w) == wl, 1.0, 0.0),
                    (0.0, 1.0))
