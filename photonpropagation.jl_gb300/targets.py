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


def module_ids(targets) -> np.ndarray:
    """module_id of each target (index i -> id), as UInt16 in the reference."""
    return np.asarray([int(getattr(t, "module_id", i + 1)) for i, t in enumerate(targets)],
                      np.uint16)
