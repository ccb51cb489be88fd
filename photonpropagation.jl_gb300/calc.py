"""Geometric times and time residuals (mirrors src/calc.jl).

Host functions with the reference's names and meaning, plus
``time_residuals_device``: the residuals of hit records in device memory
(``pp_time_residuals``), t - tgeo(module) - t0 with the module's geometric
time computed here once per module.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import check
from .medium import C_VAC_M_NS
from .sources import CherenkovTrackEmitter


def calc_tgeo(distance, medium_or_cn, target=None):
    """``calc_tgeo(distance, c_n | medium)`` and ``calc_tgeo(distance, target,
    medium)`` (src/calc.jl:24-67): distance (less the target radius) over the
    group velocity at 800 nm (or over the given speed)."""
    d = np.asarray(distance, np.float64)
    if target is not None:
        d = d - float(target.shape.radius)
    c_n = medium_or_cn if np.isscalar(medium_or_cn) else \
        float(medium_or_cn.group_velocity(800.0))
    return d / c_n


def closest_approach_distance(p0, direction, pos):
    """|(pos - p0) x dir| (src/calc.jl:69-82)."""
    a = np.asarray(pos, np.float64) - np.asarray(p0, np.float64)
    return np.linalg.norm(np.cross(a, np.asarray(direction, np.float64)), axis=-1)


def closest_approach_param(p0, direction, pos):
    """(pos - p0) . dir (src/calc.jl:186-196)."""
    a = np.asarray(pos, np.float64) - np.asarray(p0, np.float64)
    return np.sum(a * np.asarray(direction, np.float64), axis=-1)


def calc_tgeo_tracks(p0, direction, pos, medium_or_n_ph, n_grp=None, wavelength=800.0):
    """Direct Cherenkov light from a track to `pos` (src/calc.jl:118-166):
    (dir . (pos - p0) + d (n_grp n_ph - 1) / sqrt(n_ph^2 - 1)) / c, d the
    closest-approach distance; n_ph, n_grp of the medium at `wavelength`."""
    if n_grp is None:
        medium = medium_or_n_ph
        n_ph = float(medium.phase_refractive_index(wavelength))
        n_grp = C_VAC_M_NS / float(medium.group_velocity(wavelength))
    else:
        n_ph = float(medium_or_n_ph)
    dist = closest_approach_distance(p0, direction, pos)
    along = closest_approach_param(p0, direction, pos)
    return (along + dist * (n_grp * n_ph - 1.0) / np.sqrt(n_ph ** 2 - 1.0)) / C_VAC_M_NS


def shift_particle(particle, param):
    """The particle moved by `param` m along its direction, its time by
    param / c (src/calc.jl:236-247)."""
    from dataclasses import replace
    pos = np.asarray(particle.position, np.float64) + param * np.asarray(particle.direction,
                                                                         np.float64)
    return replace(particle, position=list(pos), time=particle.time + param / C_VAC_M_NS)


def shift_to_closest_approach(particle, pos):
    """The particle shifted to its closest approach to `pos` (src/calc.jl:249-265)."""
    return shift_particle(particle, float(closest_approach_param(particle.position,
                                                                 particle.direction, pos)))


def module_tgeo(setup) -> np.ndarray:
    """Geometric time of every target for the setup's first source, as
    calc_time_residual! uses it (src/calc.jl:270-323)."""
    src = setup.sources[0]
    out = np.zeros(len(setup.targets), np.float64)
    for i, t in enumerate(setup.targets):
        pos = np.asarray(t.shape.position, np.float64)
        if isinstance(src, CherenkovTrackEmitter):
            out[i] = calc_tgeo_tracks(src.position, src.direction, pos, setup.medium)
        else:
            dist = np.linalg.norm(np.asarray(src.position, np.float64) - pos)
            out[i] = calc_tgeo(dist, setup.medium, target=t)
    return out


def _residuals(table, setup, tg):
    index_of = {int(getattr(t, "module_id", i + 1)): i for i, t in enumerate(setup.targets)}
    rows = np.array([index_of[int(m)] for m in table["module_id"]], np.int64) \
        if len(table["module_id"]) else np.zeros(0, np.int64)
    table["tres"] = np.asarray(table["time"], np.float64) - tg[rows] - float(setup.sources[0].time)
    return table


def calc_time_residual_tracks(table, setup):
    """``calc_time_residual_tracks!`` (src/calc.jl:283-298): the track form for
    every module, the first source taken as the track."""
    src = setup.sources[0]
    tg = np.array([calc_tgeo_tracks(src.position, src.direction,
                                    np.asarray(t.shape.position, np.float64), setup.medium)
                   for t in setup.targets], np.float64)
    return _residuals(table, setup, tg)


def calc_time_residual_cascades(table, setup):
    """``calc_time_residual_cascades!`` (src/calc.jl:301-312)."""
    src = setup.sources[0]
    tg = np.array([calc_tgeo(np.linalg.norm(np.asarray(src.position, np.float64) -
                                            np.asarray(t.shape.position, np.float64)),
                             setup.medium, target=t) for t in setup.targets], np.float64)
    return _residuals(table, setup, tg)


def calc_time_residual(table, setup):
    """``calc_time_residual!(df, setup)``: a ``tres`` column,
    time - tgeo(module) - t0 for the first source (tracks for a
    CherenkovTrackEmitter, cascades otherwise)."""
    tg = module_tgeo(setup)
    index_of = {int(getattr(t, "module_id", i + 1)): i for i, t in enumerate(setup.targets)}
    rows = np.array([index_of[int(m)] for m in table["module_id"]], np.int64) \
        if len(table["module_id"]) else np.zeros(0, np.int64)
    t0 = float(setup.sources[0].time)
    table["tres"] = np.asarray(table["time"], np.float64) - tg[rows] - t0
    return table


def time_residuals_device(d_records: int, n: int, setup, d_tres: int, stream: int = 0) -> None:
    """Residuals of n device hit records (their module_index) into d_tres
    (float64, device), with the module geometric times of ``module_tgeo``."""
    lib = _lib.load()
    tg = np.ascontiguousarray(module_tgeo(setup), np.float64)
    check(lib.pp_time_residuals(ctypes.c_void_p(d_records), int(n),
                                tg.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(tg),
                                float(setup.sources[0].time), ctypes.c_void_p(d_tres),
                                ctypes.c_void_p(stream)), "pp_time_residuals")
