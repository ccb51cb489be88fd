"""Particles, light yields and the particle -> hits pipeline (mirrors
src/lightyield.jl:37-873 and propagate_particles, src/processing.jl:209-240).

Host-side physics that turns a particle into an emitter (its photon count is
a Poisson draw around the Cherenkov light yield) and drives the device
pipeline: propagation, time residuals, PMT detection, QE weights.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, replace
from typing import Sequence

import numpy as np
from scipy import special


from .sources import (CherenkovTrackEmitter, ExtendedCherenkovEmitter,
                      ExtendedCherenkovEmitterNoSmear, LongitudinalParameterisation,
                      PointlikeCherenkovEmitter)
from .spectrum import integrate_gauss_quad, make_cherenkov_spectrum

CASCADE_TYPES = ("EMinus", "EPlus", "Gamma", "HadronShower")
TRACK_TYPES = ("MuMinus", "MuPlus")


@dataclass
class Particle:
    """Particle(position, direction, time, energy (GeV), length (m), type)."""
    position: Sequence[float]
    direction: Sequence[float]
    time: float
    energy: float
    length: float
    type: str


def particle_shape(p: Particle) -> str:
    """'Track' for muons, 'Cascade' otherwise (PhysicsTools' particle_shape)."""
    if p.type in TRACK_TYPES:
        return "Track"
    if p.type in CASCADE_TYPES:
        return "Cascade"
    raise ValueError(f"unknown particle type {p.type}")


@dataclass(frozen=True)
class LongitudinalParametersBase:
    """Longitudinal profile parameters at 1 GeV (src/lightyield.jl:133-158)."""
    alpha: float
    beta: float
    b: float


def get_longitudinal_params(ptype: str, energy: float | None = None):
    """The type's LongitudinalParametersBase, or with `energy` (GeV) the
    energy-corrected (a, b) = (alpha + beta log10 E, b) (src/lightyield.jl:155-172)."""
    from .sources import LONGITUDINAL_PARAMETERS
    base = LongitudinalParametersBase(*LONGITUDINAL_PARAMETERS[ptype])
    if energy is None:
        return base
    return base.alpha + base.beta * math.log10(energy), base.b


@dataclass(frozen=True)
class CherenkovTrackLengthParameters:
    """alpha E^beta (and its spread alpha_dev E^beta_dev) of the Cherenkov track
    length (src/lightyield.jl:200-238)."""
    alpha: float
    beta: float
    alpha_dev: float
    beta_dev: float


class AngularEmissionProfile:
    """Marker type of the reference (src/lightyield.jl:39), no fields."""


# Cherenkov track length parametrisation, src/lightyield.jl:212-238
# (alpha, beta, alpha_dev, beta_dev) per particle type.
TRACK_LENGTH_PARAMETERS = {
    "EMinus": (5.3207078881, 1.00000211, 0.0578170887, 0.5),
    "EPlus": (5.3211320598, 0.99999254, 0.0573419669, 0.5),
    "Gamma": (5.3208540905, 0.99999877, 0.0578170887, 5.66586567),
    "HadronShower": (3.3355182722, 1.03662217, 1.1920455395, 0.80772057),
}


def cascade_cherenkov_track_length(energy: float, ptype: str) -> float:
    """alpha * E^beta (src/lightyield.jl:340-358)."""
    a, b, _, _ = TRACK_LENGTH_PARAMETERS[ptype]
    return a * energy ** b


def cascade_cherenkov_track_length_dev(energy: float, ptype: str) -> float:
    _, _, a, b = TRACK_LENGTH_PARAMETERS[ptype]
    return a * energy ** b


def rel_additional_track_length(ref_index, energy):
    """lambda + kappa log(E), lambda and kappa linear in n through the
    tabulated points at n = 1.30 and 1.36 (src/lightyield.jl:361-390)."""
    lam = 0.1842 + (ref_index - 1.30) * (0.1916 - 0.1842) / (1.36 - 1.30)
    kap = 0.0204 + (ref_index - 1.30) * (0.0207 - 0.0204) / (1.36 - 1.30)
    return lam + kap * np.log(energy)


def total_lightyield(particle: Particle, medium, spectrum) -> float:
    """Expected Cherenkov photons (src/lightyield.jl:401-435): for a cascade the
    spectrum's normalisation times the Cherenkov track length; for a track
    the integral over the spectrum of (1 + relative additional track length)
    times the track length."""
    if particle_shape(particle) == "Cascade":
        return spectrum.spectral_dist.normalization * cascade_cherenkov_track_length(
            particle.energy, particle.type)

    def integrand(wl):
        n = medium.phase_refractive_index(wl)
        return spectrum.spectrum(wl) * (1.0 + rel_additional_track_length(n, particle.energy))
    lo, hi = spectrum.wl_range
    return integrate_gauss_quad(integrand, lo, hi) * particle.length


def longitudinal_profile(z, long_param: LongitudinalParameterisation):
    """Gamma-shaped longitudinal profile at shower depth z (m), a density in
    t = z / lrad (src/lightyield.jl:259-268)."""
    t = np.asarray(z, np.float64) / long_param.lrad
    b, a = long_param.b, long_param.a
    return b * ((t * b) ** (a - 1.0) * np.exp(-(t * b)) / math.gamma(a))


def integral_long_profile(z_low, z_high, long_param: LongitudinalParameterisation):
    """Integral of the profile between two depths (src/lightyield.jl:285-298)."""
    a, b, lrad = long_param.a, long_param.b, long_param.lrad
    return special.gammainc(a, b * z_high / lrad) - special.gammainc(a, b * z_low / lrad)


def fractional_contrib_long(z_grid, long_param: LongitudinalParameterisation):
    """Fraction of the profile in each bin of z_grid, first entry 0
    (src/lightyield.jl:305-325)."""
    z = np.asarray(z_grid, np.float64)
    norm = integral_long_profile(z[0], z[-1], long_param)
    out = np.zeros_like(z)
    out[1:] = integral_long_profile(z[:-1], z[1:], long_param) / norm
    return out


# Angular distribution of cascade Cherenkov light, src/lightyield.jl:37-68
STD_ANG_DIST_PARS = (4.27033, -6.02527, 0.29887, -0.00103)


def cherenkov_ang_dist(costheta, ref_index, pars=STD_ANG_DIST_PARS):
    a, b, c, d = pars
    return a * np.exp(b * np.abs(np.asarray(costheta, np.float64) - 1.0 / ref_index) ** c) + d


def cherenkov_ang_dist_int_analytic(ref_index, lower=-1.0, upper=1.0, pars=STD_ANG_DIST_PARS):
    """The reference's closed form of the integral (src/lightyield.jl:73-111):
    on each side of the peak cos(theta_c) = 1/n the antiderivative
    (c d x + a (cc - x) Gamma(1/c, -b |x - cc|^c) (-b |x - cc|^c)^(-1/c)) / c
    with the upper incomplete gamma function, the upper branch shifted by twice
    the lower branch's value just below the peak.  That shift includes the
    d x term, so across the peak the result differs from the true integral by
    about 2 d cos(theta_c) (-0.0015 at n = 1.34); reproduced as the reference
    computes it (cherenkov_ang_dist_int_quad gives the true integral)."""
    a, b, c, d = pars
    cc = 1.0 / ref_index

    def branch(x, z):
        zz = -b * z ** c
        return (c * d * x + a * (cc - x) * special.gammaincc(1 / c, zz) * special.gamma(1 / c)
                * zz ** (-1 / c)) / c

    peak = branch(cc - 1e-5, 1e-5)

    def indef(x):
        return branch(x, cc - x) if x <= cc else branch(x, x - cc) + 2 * peak

    return indef(upper) - indef(lower)


# cherenkov_ang_dist_int(ref_index): the reference's linear interpolation of the
# closed form over [-1, 1] on n = 1.1:0.01:1.5 (src/lightyield.jl:113-130)
_ANG_INT_N = np.round(np.arange(1.1, 1.5 + 1e-9, 0.01), 10)
_ANG_INT_A = np.array([cherenkov_ang_dist_int_analytic(n) for n in _ANG_INT_N])


def cherenkov_ang_dist_int(ref_index):
    """Integral of cherenkov_ang_dist over [-1, 1] at `ref_index` in [1.1, 1.5],
    interpolated linearly as the reference's ChAngDistInt does."""
    r = np.asarray(ref_index, np.float64)
    if np.any((r < _ANG_INT_N[0] - 1e-12) | (r > _ANG_INT_N[-1] + 1e-12)):
        raise ValueError("refractive index outside the interpolation range [1.1, 1.5]")
    return np.interp(r, _ANG_INT_N, _ANG_INT_A)


def cherenkov_ang_dist_int_quad(ref_index, lower=-1.0, upper=1.0, pars=STD_ANG_DIST_PARS):
    """Integral of cherenkov_ang_dist over [lower, upper] by quadrature (an
    independent check of the closed form).  On each side of the
    peak cos(theta_c) = 1/n the substitution s = |x - 1/n|^c turns the cusp
    into the smooth integrand (a e^(b s) + d) s^(1/c - 1) / c, integrated by
    Gauss-Legendre quadrature."""
    a, b, c, d = pars
    cc = 1.0 / ref_index

    def side(length):  # integral over a distance `length` from the peak
        if length <= 0:
            return 0.0
        g = lambda u: (a * np.exp(b * u) + d) * u ** (1.0 / c - 1.0) / c  # noqa: E731
        return integrate_gauss_quad(g, 0.0, length ** c, order=100)

    def signed(x):  # integral from the peak to x (negative below the peak)
        return side(x - cc) if x >= cc else -side(cc - x)

    return signed(upper) - signed(lower)


def _poisson(mean: float, rng) -> int:
    rng = rng if rng is not None else np.random.default_rng()
    return int(rng.poisson(mean))


def extended_cherenkov_emitter(particle, medium, spectrum, oversample=1.0, rng=None,
                               no_smear=False):
    """ExtendedCherenkovEmitter(particle, medium, spectrum; oversample)
    (src/lightyield.jl:592-605): Poisson photons around the light yield."""
    lp = LongitudinalParameterisation.from_energy(particle.energy, medium, particle.type)
    n = _poisson(total_lightyield(particle, medium, spectrum) * oversample, rng)
    cls = ExtendedCherenkovEmitterNoSmear if no_smear else ExtendedCherenkovEmitter
    return cls(list(particle.position), list(particle.direction), particle.time, n, lp)


def extended_cherenkov_emitter_custom_smear(particle, medium, spectrum, cherenkov_beta_a=1.776,
                                            cherenkov_beta_b=0.164, oversample=1.0, rng=None):
    """ExtendedCherenkovEmitterCustomSmear(particle, medium, spectrum;
    cherenkov_beta_a, cherenkov_beta_b, oversample) (src/lightyield.jl:756-769)."""
    from .sources import ExtendedCherenkovEmitterCustomSmear
    lp = LongitudinalParameterisation.from_energy(particle.energy, medium, particle.type)
    n = _poisson(total_lightyield(particle, medium, spectrum) * oversample, rng)
    return ExtendedCherenkovEmitterCustomSmear(list(particle.position), list(particle.direction),
                                               particle.time, n, lp, float(cherenkov_beta_a),
                                               float(cherenkov_beta_b))


def pointlike_cherenkov_emitter(particle, medium, spectrum, rng=None):
    """PointlikeCherenkovEmitter(particle, medium, spectrum) (src/lightyield.jl:765-775)."""
    n = _poisson(total_lightyield(particle, medium, spectrum), rng)
    return PointlikeCherenkovEmitter(list(particle.position), list(particle.direction),
                                     particle.time, n)


def cherenkov_track_emitter(particle, medium, spectrum, rng=None):
    """CherenkovTrackEmitter(particle, medium, spectrum) (src/lightyield.jl:790-793)."""
    n = _poisson(total_lightyield(particle, medium, spectrum), rng)
    return CherenkovTrackEmitter(list(particle.position), list(particle.direction),
                                 particle.time, particle.length, n)


FAST_LIGHTSABRE_COEFFS = (4.9489616410707695, -2.4858046180252362, 1.1885034976827853,
                          -0.2015848374875856, 0.01626011917463439, -0.0004947317263294414)


def fast_lightsabre_muon_emitter(particle, medium, spectrum, rng=None):
    """FastLightsabreMuonEmitter (src/lightyield.jl:849-873): the bare track
    yield plus a stochastic-loss yield 10^poly(log10 E) per metre, for
    10 GeV <= E <= 1e8 GeV."""
    if not (1e1 <= particle.energy <= 1e8):
        raise ValueError("particle energy outside parametrization range")
    le = math.log10(particle.energy)
    ly_stoch = 10.0 ** sum(c * le ** i for i, c in enumerate(FAST_LIGHTSABRE_COEFFS)) * \
        particle.length
    n = _poisson(total_lightyield(particle, medium, spectrum) + ly_stoch, rng)
    return CherenkovTrackEmitter(list(particle.position), list(particle.direction),
                                 particle.time, particle.length, n)


FastLightsabreMuonEmitter = fast_lightsabre_muon_emitter  # the reference's constructor name


def split_source(source, parts: int):
    """The source as `parts` copies sharing its photons, the last one taking
    the remainder (src/lightyield.jl:440-472)."""
    if source.photons < parts:
        raise ValueError("Cannot split source. Fewer photons than parts")
    q, r = divmod(int(source.photons), parts)
    return [replace(copy.copy(source), photons=q + (r if i == parts - 1 else 0))
            for i in range(parts)]


def rescale_source(source, factor: float):
    """A copy with ceil(photons * factor) photons (src/lightyield.jl:480-490)."""
    return replace(copy.copy(source), photons=int(math.ceil(source.photons * factor)))


def propagate_particles(particles, targets, seed, medium, rng=None, device=0):
    """``propagate_particles(particles, targets, seed, medium)``
    (src/processing.jl:209-240): cascades become ExtendedCherenkovEmitters and
    muons FastLightsabreMuonEmitters over a 300-800 nm Cherenkov spectrum;
    propagation, time residuals, PMT hits and QE weights follow.  Returns
    the hit table, or None when no photon reached a module."""
    from .calc import calc_time_residual
    from .detection import calc_pe_weight, make_hits_from_photons
    from .processing import propagate_photons
    from .propsetup import PhotonPropSetup
    spectrum = make_cherenkov_spectrum((300.0, 800.0), medium)
    srcs = [extended_cherenkov_emitter(p, medium, spectrum, rng=rng)
            if particle_shape(p) == "Cascade" else
            fast_lightsabre_muon_emitter(p, medium, spectrum, rng=rng) for p in particles]
    setup = PhotonPropSetup(srcs, list(targets), medium, spectrum, seed)
    photons = propagate_photons(setup, device=device)
    if photons.nrow == 0:
        return None
    calc_time_residual(photons, setup)
    hits = make_hits_from_photons(photons, setup, seed=seed, device=device)
    return calc_pe_weight(hits, setup)



