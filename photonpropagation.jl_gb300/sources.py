"""Photon sources (mirrors PhotonPropagation.jl src/lightyield.jl:437-873).

Each emitter converts to the 80-byte ``pp_source`` record of the C ABI.
Field names and order follow the reference structs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Sequence, Tuple

import numpy as np

from . import _lib


def _vec3(v) -> Tuple[float, float, float]:
    a = np.asarray(v, np.float32).reshape(3)
    return (float(a[0]), float(a[1]), float(a[2]))


@dataclass
class LongitudinalParameterisation:
    """Gamma-profile parameters of a cascade (src/lightyield.jl:175-197)."""
    a: float
    b: float
    lrad: float

    @classmethod
    def from_energy(cls, energy: float, medium, ptype: str = "EMinus"):
        """a = alpha + beta*log10(E), b, lrad = X0/rho*10 (src/lightyield.jl:164-197)."""
        alpha, beta, b = LONGITUDINAL_PARAMETERS[ptype]
        lrad = medium.radiation_length() / medium.material_density() * 10.0
        return cls(alpha + beta * math.log10(energy), b, lrad)


# src/lightyield.jl:148-151 (alpha, beta, b) per particle type
LONGITUDINAL_PARAMETERS = {
    "EMinus": (2.01849, 1.45469, 0.63207),
    "EPlus": (2.00035, 1.45501, 0.63008),
    "Gamma": (2.83923, 1.34031, 0.64526),
    "HadronShower": (1.58357, 0.96448, 0.33833),
}


class PhotonSource:
    kind: int
    photons: int

    def to_record(self) -> _lib.pp_source:
        raise NotImplementedError

    def _base(self) -> _lib.pp_source:
        r = _lib.pp_source()
        r.kind = self.kind
        r.photons = int(self.photons)
        # Optional photon-range offset (set as a plain attribute): the source
        # then emits photons first_photon .. first_photon + n - 1.
        r.first_photon = int(getattr(self, "first_photon", 0))
        return r


@dataclass
class PointlikeIsotropicEmitter(PhotonSource):
    """src/lightyield.jl:549-553; initial state src/photon_prop_cuda.jl:158-163."""
    position: Sequence[float]
    time: float
    photons: int
    kind = _lib.PP_SRC_POINTLIKE_ISOTROPIC

    def to_record(self):
        r = self._base()
        r.position[:] = _vec3(self.position)
        r.time = float(self.time)
        return r


@dataclass
class PointlikeTimeRangeEmitter(PhotonSource):
    """src/lightyield.jl:592-596; src/photon_prop_cuda.jl:165-171."""
    position: Sequence[float]
    time_range: Tuple[float, float]
    photons: int
    kind = _lib.PP_SRC_POINTLIKE_TIME_RANGE

    def to_record(self):
        r = self._base()
        r.position[:] = _vec3(self.position)
        r.time = float(self.time_range[0])
        r.time_end = float(self.time_range[1])
        return r


@dataclass
class CollimatedIsotropicEmitter(PhotonSource):
    """src/lightyield.jl:570-575; src/photon_prop_cuda.jl:186-195."""
    position: Sequence[float]
    time: float
    photons: int
    cut_angle_cos: float
    kind = _lib.PP_SRC_COLLIMATED_ISOTROPIC

    def to_record(self):
        r = self._base()
        r.position[:] = _vec3(self.position)
        r.time = float(self.time)
        r.cut_angle_cos = float(self.cut_angle_cos)
        return r


@dataclass
class PencilEmitter(PhotonSource):
    """src/lightyield.jl:527-534; src/photon_prop_cuda.jl:197-208."""
    position: Sequence[float]
    direction: Sequence[float]
    beam_divergence: float
    time: float
    photons: int
    kind = _lib.PP_SRC_PENCIL

    def to_record(self):
        r = self._base()
        r.position[:] = _vec3(self.position)
        r.direction[:] = _vec3(self.direction)
        r.beam_divergence = float(self.beam_divergence)
        r.time = float(self.time)
        return r


@dataclass
class AxiconeEmitter(PhotonSource):
    """src/lightyield.jl:503-510; src/photon_prop_cuda.jl:173-184."""
    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    angle: float
    beam_divergence: float
    kind = _lib.PP_SRC_AXICONE

    def to_record(self):
        r = self._base()
        r.position[:] = _vec3(self.position)
        r.direction[:] = _vec3(self.direction)
        r.time = float(self.time)
        r.angle = float(self.angle)
        r.beam_divergence = float(self.beam_divergence)
        return r


class _CherenkovBase(PhotonSource):
    def _cher(self, r):
        r.position[:] = _vec3(self.position)
        r.direction[:] = _vec3(self.direction)
        r.time = float(self.time)
        return r


@dataclass
class ExtendedCherenkovEmitter(_CherenkovBase):
    """Cascade with a gamma longitudinal profile and a smeared Cherenkov cone
    (src/lightyield.jl:616-622; src/photon_prop_cuda.jl:211-222)."""
    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    long_param: LongitudinalParameterisation
    kind = _lib.PP_SRC_EXTENDED_CHERENKOV

    def to_record(self):
        r = self._cher(self._base())
        r.long_a = float(self.long_param.a)
        r.long_b = float(self.long_param.b)
        r.long_lrad = float(self.long_param.lrad)
        return r


@dataclass
class ExtendedCherenkovEmitterNoSmear(ExtendedCherenkovEmitter):
    """All photons exactly on the Cherenkov cone (src/lightyield.jl:670-676;
    src/photon_prop_cuda.jl:225-236)."""
    kind = _lib.PP_SRC_EXTENDED_CHERENKOV_NOSMEAR


@dataclass
class ExtendedCherenkovEmitterCustomSmear(ExtendedCherenkovEmitter):
    """The cascade emitter with the track direction's cos(theta) drawn as
    2 Beta(cherenkov_beta_a, cherenkov_beta_b) - 1 (src/lightyield.jl:725-769;
    src/photon_prop_cuda.jl:134-154, 238-250).  The device samples it from a
    quantile table of that Beta distribution (one table per distinct (a, b),
    pp_set_track_smear_tables)."""
    cherenkov_beta_a: float = 1.776
    cherenkov_beta_b: float = 0.164


@dataclass
class PointlikeCherenkovEmitter(_CherenkovBase):
    """src/lightyield.jl PointlikeCherenkovEmitter; src/photon_prop_cuda.jl:254-263."""
    position: Sequence[float]
    direction: Sequence[float]
    time: float
    photons: int
    kind = _lib.PP_SRC_POINTLIKE_CHERENKOV

    def to_record(self):
        return self._cher(self._base())


@dataclass
class CherenkovTrackEmitter(_CherenkovBase):
    """Uniform emission along a track of `length` m (src/photon_prop_cuda.jl:265-276)."""
    position: Sequence[float]
    direction: Sequence[float]
    time: float
    length: float
    photons: int
    kind = _lib.PP_SRC_CHERENKOV_TRACK

    def to_record(self):
        r = self._cher(self._base())
        r.length = float(self.length)
        return r


TRACK_SMEAR_KINDS = (_lib.PP_SRC_EXTENDED_CHERENKOV, _lib.PP_SRC_POINTLIKE_CHERENKOV,
                     _lib.PP_SRC_CHERENKOV_TRACK)


def to_records(sources) -> "ctypes.Array":
    arr = (_lib.pp_source * max(1, len(sources)))()
    for i, s in enumerate(sources):
        arr[i] = s.to_record()
    return arr


def source_photons(photons: int, scaling: float) -> int:
    """floor(Float32(photons) * Float32(scaling)) in FP32 (src/photon_prop_cuda.jl:456)."""
    x = np.float32(photons) * np.float32(scaling)
    return int(np.floor(x)) if x > 0 else 0
