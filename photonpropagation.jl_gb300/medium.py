"""Media of the photon-transport path, evaluated on the host into tables.

Mirrors PhotonPropagation.jl's ``CascadiaMediumProperties``
(src/water_properties.jl:43-100) and ``SimpleMediumProperties``
(src/simple_medium.jl:1-15).  The kernel reads per-wavelength tables of
scattering length, group velocity, absorption length and phase refractive
index (linear interpolation on a fine uniform grid) plus the MixedHGES phase
function parameters.

The Cascadia formulas live in CherenkovMediumBase 1.0.0, which is not part of
the reference tree; they are restated here from their published forms:
Kopelevich scattering (pure water + small + large particles), Quan & Fry
(1995) sea-water index with a linear pressure term, group velocity
``c / (n - (n*wl) * dn/dwl)``, and linear interpolation of the STRAW
absorption-length fit (the reference's own asset table).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib

C_VAC_M_NS = 0.299792458

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                     "attenuation_length_straw_fit.csv")

# src/water_properties.jl:33-41
CASCADIA_ES_B = 0.835
CASCADIA_VOL_CONC_SMALL_PART = 7.5e-3
CASCADIA_VOL_CONC_LARGE_PART = 7.5e-3
CASCADIA_HG_G = 0.95
CASCADIA_SALINITY = 34.82  # permille
CASCADIA_TEMPERATURE = 1.8  # C
CASCADIA_PRESSURE = 265.917473476  # atm
CASCADIA_RADIATION_LENGTH = 36.08  # g/cm^2


def dippr105(temperature_k: float, A=0.14395, B=0.0112, C=649.727, D=0.05107) -> float:
    """DIPPR-105 liquid density correlation for water (kg/m^3)."""
    return A / B ** (1.0 + (1.0 - temperature_k / C) ** D)


CASCADIA_DENSITY = dippr105(CASCADIA_TEMPERATURE + 273.15)


def load_abs_table():
    wl, al = [], []
    with open(_DATA) as f:
        for line in f:
            if line.startswith("#") or not line.strip():
                continue
            a, b = line.split(",")
            wl.append(float(a))
            al.append(float(b))
    return np.asarray(wl, np.float64), np.asarray(al, np.float64)


@dataclass
class MediumTables:
    """Per-wavelength tables handed to the device (float32)."""
    wl_min: float
    wl_step: float
    scattering_length: np.ndarray
    group_velocity: np.ndarray
    absorption_length: np.ndarray
    phase_refractive_index: np.ndarray
    hg_g: float
    es_b: float
    hg_weight: float
    phase_kind: int = 0  # PP_PHASE_HG_ES / PP_PHASE_HG_SL

    @property
    def n_knots(self) -> int:
        return int(self.scattering_length.shape[0])


class MediumProperties:
    """Common interface (CherenkovMediumBase's MediumProperties)."""

    hg_g: float
    es_b: float
    hg_weight: float

    def scattering_length(self, wl):
        raise NotImplementedError

    def group_velocity(self, wl):
        raise NotImplementedError

    def absorption_length(self, wl):
        raise NotImplementedError

    def phase_refractive_index(self, wl):
        raise NotImplementedError

    def cherenkov_angle(self, wl):
        return np.arccos(1.0 / np.asarray(self.phase_refractive_index(wl), np.float64))

    def mean_scattering_angle(self) -> float:
        """Mean cosine of the phase-function mixture (ES is symmetric)."""
        return self.hg_weight * self.hg_g

    def tables(self, wl_lo: float, wl_hi: float, step: float = 0.125) -> MediumTables:
        """Tables on [wl_lo, wl_hi] (padded by one step) with knots every `step` nm.
        The knots fall on multiples of `step`, so the 5 nm absorption table
        knots are reproduced exactly by the linear interpolation."""
        lo = math.floor(wl_lo / step) * step - step
        hi = math.ceil(wl_hi / step) * step + step
        n = int(round((hi - lo) / step)) + 1
        wl = lo + step * np.arange(n, dtype=np.float64)
        return MediumTables(
            wl_min=float(lo), wl_step=float(step),
            scattering_length=np.asarray(self.scattering_length(wl), np.float32),
            group_velocity=np.asarray(self.group_velocity(wl), np.float32),
            absorption_length=np.asarray(self.absorption_length(wl), np.float32),
            phase_refractive_index=np.asarray(self.phase_refractive_index(wl), np.float32),
            hg_g=float(self.hg_g), es_b=float(self.es_b), hg_weight=float(self.hg_weight),
            phase_kind=int(getattr(self, "phase_kind", 0)))

    def oracle_params(self) -> dict:
        raise NotImplementedError


class CascadiaMediumProperties(MediumProperties):
    """Cascadia Basin sea water (src/water_properties.jl:43-100).

    ``CascadiaMediumProperties(hg_g, pure_water_fraction, abs_scale, sca_scale)``
    as in the reference; ``CascadiaMediumProperties()`` gives the reference's
    defaults (0.95, 0.2, 1, 1) and, unlike v0.9.3, the README's one-argument
    form ``CascadiaMediumProperties(0.95)`` is accepted too.

    Phase function: ``MixedHGES(hg_g, 0.835, 1 - pure_water_fraction)``; the
    third parameter is read as the probability of the Henyey-Greenstein
    (particle) component, the rest being Einstein-Smoluchowski (pure water).
    """

    def __init__(self, hg_g: float = CASCADIA_HG_G, pure_water_fraction: float = 0.2,
                 abs_scale: float = 1.0, sca_scale: float = 1.0):
        self.hg_g = float(np.float32(hg_g))
        self.pure_water_fraction = float(np.float32(pure_water_fraction))
        self.abs_scale = float(np.float32(abs_scale))
        self.sca_scale = float(np.float32(sca_scale))
        self.es_b = CASCADIA_ES_B
        self.hg_weight = float(np.float32(1.0) - np.float32(pure_water_fraction))
        self.vol_conc_small = CASCADIA_VOL_CONC_SMALL_PART
        self.vol_conc_large = CASCADIA_VOL_CONC_LARGE_PART
        self.salinity = CASCADIA_SALINITY
        self.temperature = CASCADIA_TEMPERATURE
        self.pressure = CASCADIA_PRESSURE
        self._abs_wl, self._abs_len = load_abs_table()

    # -- Kopelevich scattering ---------------------------------------------
    def scattering_coefficient(self, wl):
        x = 550.0 / np.asarray(wl, np.float64)
        return (0.0017 * x ** 4.3 + 1.34 * self.vol_conc_small * x ** 1.7 +
                0.312 * self.vol_conc_large * x ** 0.3)

    def scattering_length(self, wl):
        return 1.0 / self.scattering_coefficient(wl) * self.sca_scale

    # -- Quan & Fry dispersion -------------------------------------------------
    def phase_refractive_index(self, wl):
        S, T, P = self.salinity, self.temperature, self.pressure
        x = 1.0 / np.asarray(wl, np.float64)
        return (1.31405 + 1.45e-5 * P + (1.779e-4 - 1.05e-6 * T + 1.6e-8 * T * T) * S
                - 2.02e-6 * T * T + (15.868 + 0.01155 * S - 0.00423 * T) * x
                - 4382.0 * x * x + 1.1455e6 * x ** 3)

    def dispersion(self, wl):
        """dn/dwl (1/nm)."""
        S, T = self.salinity, self.temperature
        x = 1.0 / np.asarray(wl, np.float64)
        return (-(15.868 + 0.01155 * S - 0.00423 * T) * x * x + 2.0 * 4382.0 * x ** 3
                - 3.0 * 1.1455e6 * x ** 4)

    def group_refractive_index(self, wl):
        n = self.phase_refractive_index(wl)
        return n - n * np.asarray(wl, np.float64) * self.dispersion(wl)

    def group_velocity(self, wl):
        return C_VAC_M_NS / self.group_refractive_index(wl)

    # -- absorption --------------------------------------------------------------
    def absorption_length(self, wl):
        return np.interp(np.asarray(wl, np.float64), self._abs_wl, self._abs_len) * self.abs_scale

    def radiation_length(self) -> float:
        return CASCADIA_RADIATION_LENGTH

    def material_density(self) -> float:
        return CASCADIA_DENSITY

    def oracle_params(self) -> dict:
        return dict(kind=0, hg_g=self.hg_g, es_b=self.es_b, hg_weight=self.hg_weight,
                    abs_scale=self.abs_scale, sca_scale=self.sca_scale,
                    vol_conc_small=self.vol_conc_small, vol_conc_large=self.vol_conc_large,
                    salinity=self.salinity, temperature=self.temperature,
                    pressure=self.pressure, abs_wl=self._abs_wl, abs_len=self._abs_len)


@dataclass
class SimpleMediumProperties(MediumProperties):
    """Constant-property medium with pure Henyey-Greenstein scattering
    (src/simple_medium.jl:1-15)."""
    absorption_length_m: float = 30.0
    scattering_length_m: float = 50.0
    phase_refractive_index_value: float = 1.35
    mean_scattering_angle_value: float = 0.95
    group_velocity_m_ns: float = 0.2
    es_b: float = field(default=CASCADIA_ES_B)

    def __post_init__(self):
        self.hg_g = float(self.mean_scattering_angle_value)
        self.hg_weight = 1.0

    def scattering_length(self, wl):
        return np.full(np.shape(wl), self.scattering_length_m, np.float64)

    def group_velocity(self, wl):
        return np.full(np.shape(wl), self.group_velocity_m_ns, np.float64)

    def absorption_length(self, wl):
        return np.full(np.shape(wl), self.absorption_length_m, np.float64)

    def phase_refractive_index(self, wl):
        return np.full(np.shape(wl), self.phase_refractive_index_value, np.float64)

    def oracle_params(self) -> dict:
        return dict(kind=1, hg_g=self.hg_g, es_b=self.es_b, hg_weight=1.0,
                    s_sca_len=self.scattering_length_m, s_abs_len=self.absorption_length_m,
                    s_ref_index=self.phase_refractive_index_value,
                    s_group_velocity=self.group_velocity_m_ns)


class HomogenousIceProperties(MediumProperties):
    """Deep homogeneous ice with the SPICE model (src/ice_properties.jl:26-176).

    ``HomogenousIceProperties(radiation_length=..., mean_scattering_angle=...,
    hg_fraction=..., A_SPICE=..., B_SPICE=..., D_SPICE=..., E_SPICE=...,
    a_dust_400=..., b_dust_400=..., alpha_sca_dust=..., kappa_abs_dust=...,
    deltaTSPICE=..., abs_scale=..., sca_scale=...)`` with the reference's keyword
    names (stored as FP32, the device's precision).  Phase function:
    Henyey-Greenstein at the mean cosine g with probability ``hg_fraction``,
    else simplified Liu at g (cos = 2 u^((1-g)/(1+g)) - 1), the mixture of
    ``mixed_hg_sl_scattering_func_ppc`` (CherenkovMediumBase 1.0.0, absent
    here) with ``hg_fraction`` read as the HG weight, as the field's docstring
    says.  Both components have mean cosine g."""

    phase_kind = _lib.PP_PHASE_HG_SL
    es_b = 0.0

    def __init__(self, radiation_length, mean_scattering_angle, hg_fraction, A_SPICE, B_SPICE,
                 D_SPICE, E_SPICE, a_dust_400, b_dust_400, alpha_sca_dust, kappa_abs_dust,
                 deltaTSPICE, abs_scale=1.0, sca_scale=1.0):
        f32 = lambda x: float(np.float32(x))  # noqa: E731
        self.radiation_length_gcm2 = f32(radiation_length)
        self.hg_g = f32(mean_scattering_angle)
        self.hg_weight = f32(hg_fraction)
        self.A_SPICE, self.B_SPICE = f32(A_SPICE), f32(B_SPICE)
        self.D_SPICE, self.E_SPICE = f32(D_SPICE), f32(E_SPICE)
        self.a_dust_400, self.b_dust_400 = f32(a_dust_400), f32(b_dust_400)
        self.alpha_sca_dust, self.kappa_abs_dust = f32(alpha_sca_dust), f32(kappa_abs_dust)
        self.deltaTSPICE = f32(deltaTSPICE)
        self.abs_scale, self.sca_scale = f32(abs_scale), f32(sca_scale)

    def mean_scattering_angle(self) -> float:
        return self.hg_g

    def radiation_length(self) -> float:
        return self.radiation_length_gcm2

    def material_density(self) -> float:
        return 0.910 * 1000  # src/ice_properties.jl:91

    def phase_refractive_index(self, wl):
        """Polynomial in wl/1000 (src/ice_properties.jl:98-107)."""
        x = np.asarray(wl, np.float64) / 1000.0
        return 1.55749 - 1.57988 * x + 3.99993 * x ** 2 - 4.68271 * x ** 3 + 2.09354 * x ** 4

    def group_refractive_index(self, wl):
        """n times a second polynomial in wl/1000 (src/ice_properties.jl:110-121)."""
        x = np.asarray(wl, np.float64) / 1000.0
        return self.phase_refractive_index(wl) * (1 + 0.227106 - 0.954648 * x + 1.42568 * x ** 2
                                                  - 0.711832 * x ** 3)

    def group_velocity(self, wl):
        return C_VAC_M_NS / self.group_refractive_index(wl)

    def absorption_length(self, wl):
        """1 / (a_dust (wl/400)^-kappa + A exp(-B/wl) (1 + 0.01 dT)), scaled
        (src/ice_properties.jl:131-160)."""
        wl = np.asarray(wl, np.float64)
        a = (self.a_dust_400 * (wl / 400.0) ** (-self.kappa_abs_dust) +
             self.A_SPICE * np.exp(-self.B_SPICE / wl) * (1 + 0.01 * self.deltaTSPICE))
        return 1.0 / a * self.abs_scale

    def scattering_length(self, wl):
        """(1 - g) / (b_dust (wl/400)^-alpha), scaled (src/ice_properties.jl:162-174)."""
        wl = np.asarray(wl, np.float64)
        eff = self.b_dust_400 * (wl / 400.0) ** (-self.alpha_sca_dust)
        return 1.0 / (eff / (1 - self.hg_g)) * self.sca_scale

    def oracle_params(self) -> dict:
        return dict(kind=2, hg_g=self.hg_g, es_b=0.0, hg_weight=self.hg_weight,
                    abs_scale=self.abs_scale, sca_scale=self.sca_scale,
                    i_a_dust_400=self.a_dust_400, i_b_dust_400=self.b_dust_400,
                    i_alpha_sca_dust=self.alpha_sca_dust, i_kappa_abs_dust=self.kappa_abs_dust,
                    i_A=self.A_SPICE, i_B=self.B_SPICE, i_delta_t=self.deltaTSPICE,
                    i_mean_cos=self.hg_g, phase_kind=int(_lib.PP_PHASE_HG_SL))


def make_homogenous_clearice_properties(T=None, abs_scale=1.0, sca_scale=1.0):
    """The "homogeneous clear ice" model (src/ice_properties.jl:49-64); the
    element type T of the reference is accepted and ignored (FP32 on the device)."""
    return HomogenousIceProperties(
        radiation_length=39.652 / 0.9216, mean_scattering_angle=0.9, hg_fraction=0.45,
        A_SPICE=6954.090332031250, B_SPICE=6617.754394531250, D_SPICE=0.0, E_SPICE=0.0,
        a_dust_400=0.006350013, b_dust_400=0.02331206666666667, alpha_sca_dust=0.898608505726,
        kappa_abs_dust=1.084106802940, deltaTSPICE=12.115215000000001, abs_scale=abs_scale,
        sca_scale=sca_scale)

