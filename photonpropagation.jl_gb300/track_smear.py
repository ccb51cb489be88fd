"""Direction of the charged-particle track about a cascade axis.

The reference samples it with ``sample_cherenkov_track_direction``
(PhysicsTools 0.8.2, absent from the reference tree; called at
src/photon_prop_cuda.jl:89, :123).  Its sibling emitter
``ExtendedCherenkovEmitterCustomSmear`` (src/lightyield.jl) draws
``cos(theta) = 2 * Beta(a, b) - 1`` with defaults a = 1.776, b = 0.164; that
Beta law is the default here.  The device samples a quantile table of
cos(theta) (``pp_set_track_smear``): a Julia host may instead fill the table
from many draws of the reference's own function.
"""
from __future__ import annotations

import numpy as np

DEFAULT_BETA_A = 1.776
DEFAULT_BETA_B = 0.164
DEFAULT_KNOTS = 4096


def beta_track_quantiles(a: float = DEFAULT_BETA_A, b: float = DEFAULT_BETA_B,
                         n: int = DEFAULT_KNOTS) -> np.ndarray:
    """Quantiles of cos(theta) = 2 Beta(a, b) - 1 at u = i / (n - 1)."""
    from scipy.special import betaincinv
    u = np.linspace(0.0, 1.0, n)
    x = betaincinv(a, b, u)
    return np.clip(2.0 * x - 1.0, -1.0, 1.0).astype(np.float32)


def empirical_quantiles(cos_samples, n: int = DEFAULT_KNOTS) -> np.ndarray:
    """Quantile table from samples of cos(theta) (e.g. drawn with the reference's
    own sample_cherenkov_track_direction)."""
    c = np.sort(np.asarray(cos_samples, np.float64))
    return np.clip(np.quantile(c, np.linspace(0.0, 1.0, n)), -1.0, 1.0).astype(np.float32)
