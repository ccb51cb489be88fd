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


@dataclass
class DetectorLine:
    """DetectorLine(x_pos, y_pos, radius, targets) (src/photon_prop_cuda.jl:418-423):
    a vertical line at (x_pos, y_pos) whose module shapes lie within `radius`
    of it in the xy plane."""
    x_pos: float
    y_pos: float
    radius: float
    targets: Sequence


@dataclass
class DetectorLines:
    """DetectorLines(lines) (src/photon_prop_cuda.jl:425-427): lines with the
    same number of modules each, searched line by line in the kernel.  Not
    iterable, as in the reference."""
    lines: Sequence[DetectorLine]

    def __post_init__(self):
        self.lines = list(self.lines)
        if not self.lines:
            raise ValueError("DetectorLines needs at least one line")
        n = len(self.lines[0].targets)
        if n < 1 or any(len(line.targets) != n for line in self.lines):
            raise ValueError("every DetectorLine must hold the same number (>= 1) of modules")

    @property
    def modules_per_line(self) -> int:
        return len(self.lines[0].targets)


def record_count(targets) -> int:
    """Number of pp_target records for `targets` (a line adds one record)."""
    if isinstance(targets, DetectorLines):
        return len(targets.lines) * (targets.modules_per_line + 1)
    return len(targets)


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
    """True when a target is not a sphere or the targets are detector lines
    (then the targets are tested at every step in order, with no culling
    grid)."""
    if isinstance(targets, DetectorLines):
        return True
    return any(not isinstance(getattr(t, "shape", t), Spherical) for t in targets)


def to_targets(targets) -> "_lib.pp_target array":
    """pp_target records (any shape) in index order; detector lines as one
    PP_TARGET_LINE record followed by the line's modules, line by line."""
    if isinstance(targets, DetectorLines):
        n = targets.modules_per_line
        arr = (_lib.pp_target * record_count(targets))()
        for li, line in enumerate(targets.lines):
            head = arr[li * (n + 1)]
            head.position[:] = (float(np.float32(line.x_pos)), float(np.float32(line.y_pos)), 0.0)
            head.radius = float(np.float32(line.radius))
            head.kind = _lib.PP_TARGET_LINE
            head.reserved = n
            mods = to_targets(list(line.targets))
            for m in range(n):
                arr[li * (n + 1) + 1 + m] = mods[m]
        return arr
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
    if isinstance(targets, DetectorLines):
        # src/processing.jl:67 iterates setup.targets, which DetectorLines does not support
        raise TypeError("DetectorLines has no module ids to map: propagate_photons fails on it "
                        "as in the reference; run_photon_prop_no_local_cache returns the "
                        "kernel's module index t + N * line")
    return np.asarray([int(getattr(t, "module_id", i + 1)) for i, t in enumerate(targets)],
                      np.uint16)


def check_intersection(shape, pos, direction, step):
    """``check_intersection(shape, pos, dir, step)`` (src/photon_prop_cuda.jl:309-404),
    host form in FP32 as the device evaluates it: (hit, distance) for a sphere
    (the near root strictly inside (0, step)), a horizontal rectangle or a
    disc (met at d = (z_s - z) / dir_z in [0, step], strictly inside)."""
    f = np.float32
    p = np.asarray(pos, f)
    d = np.asarray(direction, f)
    L = f(step)
    c = np.asarray(shape.position, f)
    if isinstance(shape, Spherical):
        dp = (p - c).astype(f)
        a = f(np.dot(d, dp))
        b = f(a * a - (f(np.dot(dp, dp)) - f(shape.radius) * f(shape.radius)))
        dist = f(-a - np.sqrt(abs(b))) if b >= 0 else f(-1)
        return (True, float(dist)) if (dist > 0 and dist < L) else (False, float("nan"))
    if d[2] == 0:
        return False, float("nan")
    dist = f((c[2] - p[2]) / d[2])
    if dist < 0 or dist > L:
        return False, float("nan")
    x, y = f(p[0] + d[0] * dist - c[0]), f(p[1] + d[1] * dist - c[1])
    if isinstance(shape, Rectangular):
        inside = abs(x) < f(0.5) * f(shape.length_x) and abs(y) < f(0.5) * f(shape.length_y)
    elif isinstance(shape, Circular):
        inside = x * x + y * y < f(shape.radius) * f(shape.radius)
    else:
        raise TypeError(f"no intersection test for {type(shape).__name__}")
    return (True, float(dist)) if inside else (False, float("nan"))

