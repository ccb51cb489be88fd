"""Targets (mirrors NeutrinoTelescopeBase's Spherical / HomogeneousDetector as
used by PhotonPropagation.jl, README.md example and src/processing.jl:61-70)."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib


@dataclass
class Spherical:
    """Spherical{Float32} target shape: position (m) and radius (m)."""
    position: Sequence[float]
    radius: float


@dataclass
class Rectangular:
    """Horizontal rectangle (normal e_z) centred at `position`, sides
    length_x, length_y (src/photon_prop_cuda.jl:353-378)."""
    position: Sequence[float]
    length_x: float
    length_y: float


@dataclass
class Circular:
    """Horizontal disc (normal e_z) centred at `position` (src/photon_prop_cuda.jl:380-404)."""
    position: Sequence[float]
    radius: float


@dataclass
class HomogeneousDetector:
    """A detector module: its shape, active area (m^2) and UInt16 module id."""
    shape: Spherical
    pmt_area: float
    module_id: int


def to_spheres(targets) -> "_lib.pp_sphere array":
    arr = (_lib.pp_sphere * max(1, len(targets)))()
    for i, t in enumerate(targets):
        shape = t.shape if hasattr(t, "shape") else t
        if not isinstance(shape, Spherical):
            raise TypeError(f"target {i}: only Spherical shapes are supported (got {type(shape)})")
        p = np.asarray(shape.position, np.float32).reshape(3)
        arr[i].position[:] = (float(p[0]), float(p[1]), float(p[2]))
        arr[i].radius = float(np.float32(shape.radius))
    return arr


def is_shaped(targets) -> bool:
    """True when a target is not a sphere (then every target is tested at
    every step, with no culling grid)."""
    return any(not isinstance(getattr(t, "shape", t), Spherical) for t in targets)


def to_targets(targets) -> "_lib.pp_target array":
    """pp_target records (any shape) in index order."""
    arr = (_lib.pp_target * max(1, len(targets)))()
    for i, t in enumerate(targets):
        shape = getattr(t, "shape", t)
        p = np.asarray(shape.position, np.float32).reshape(3)
        arr[i].position[:] = (float(p[0]), float(p[1]), float(p[2]))
        if isinstance(shape, Spherical):
            arr[i].kind = _lib.PP_TARGET_SPHERE
            arr[i].radius = float(np.float32(shape.radius))
        elif isinstance(shape, Rectangular):
            arr[i].kind = _lib.PP_TARGET_RECTANGLE
            arr[i].length_x = float(np.float32(shape.length_x))
            arr[i].length_y = float(np.float32(shape.length_y))
        elif isinstance(shape, Circular):
            arr[i].kind = _lib.PP_TARGET_DISC
            arr[i].radius = float(np.float32(shape.radius))
        else:
            raise TypeError(f"target {i}: unsupported shape {type(shape).__name__}")
    return arr


def module_ids(targets) -> np.ndarray:
    """module_id of each target (index i -> id), as UInt16 in the reference."""
    return np.asarray([int(getattr(t, "module_id", i + 1)) for i, t in enumerate(targets)],
                      np.uint16)
