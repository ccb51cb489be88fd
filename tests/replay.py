"""Photon-by-photon comparison of two hit tables (replay parity).

Both tables hold the hits of the same photons (keyed by (source, photon)).
The reference's ray-sphere formula d = -a - sqrt(a^2 - (|p-c|^2 - r^2)) is
ill-conditioned at grazing incidence: an FP32 rounding of size eps in
a^2 or |p-c|^2 moves d by about eps * L^2 / (2 r cos_inc), L the distance from
the step start to the sphere.  The position tolerance therefore has a
relative part (1e-5) and a conditioning part; directions, wavelengths, step
counts and module indices are compared without it.
"""
import numpy as np

EPS32 = 2.0 ** -24


def _key(t):
    return np.asarray(t["source_index"], np.int64) * (1 << 40) + np.asarray(t["photon_index"],
                                                                           np.int64)


def cos_incidence(pos, direction, centers, radii):
    n = (pos - centers) / radii[:, None]
    return np.abs(np.sum(n * direction, axis=1))


MODES = {
    # replay kernel (IEEE math, no contraction) vs the FP32 oracle
    "precise": dict(rel=1e-5, grazing_cos=0.02, min_match=0.999, max_nongrazing=0.001),
    # fast kernel (SFU approximations): the reference's sqrt(1 - c^2) amplifies
    # 1-ulp differences of forward scattering cosines, so trajectories drift
    # apart along the path (measured p99 of the relative position error 9e-6
    # on C0, 1.3e-4 on C1, all within 5e-4) and a few percent of the hits may
    # differ (C1: 11 one-sided of 310, balanced 6 : 5)
    "fast": dict(rel=1e-3, grazing_cos=0.02, min_match=0.95, max_nongrazing=0.05),
    # FP32 vs FP64 oracle: the same amplification of FP32 rounding
    "f32_vs_f64": dict(rel=2e-3, grazing_cos=0.02, min_match=0.95, max_nongrazing=0.05),
}


def compare(got, want, spheres_xyzr, mode="precise", cond_factor=16.0, rel=None):
    cfg = dict(MODES[mode])
    if rel is not None:
        cfg["rel"] = rel
    return _compare(got, want, spheres_xyzr, cond_factor=cond_factor, **cfg)


def _compare(got, want, spheres_xyzr, rel, grazing_cos, min_match, max_nongrazing,
             cond_factor):
    """got/want: column dicts (position (n,3), direction, initial_direction,
    wavelength, time, dist_travelled, module_index (1-based), n_steps,
    photon_index, source_index).  spheres_xyzr: (n_targets, 4).
    Returns a dict of statistics; raises AssertionError on a mismatch."""
    kg, kw = _key(got), _key(want)
    assert len(np.unique(kg)) == len(kg), "duplicate photon in got"
    assert len(np.unique(kw)) == len(kw), "duplicate photon in want"
    common, ig, iw = np.intersect1d(kg, kw, return_indices=True)
    only_g = np.setdiff1d(np.arange(len(kg)), ig)
    only_w = np.setdiff1d(np.arange(len(kw)), iw)
    sph = np.asarray(spheres_xyzr, np.float64)

    def cos_of(t, idx):
        if len(idx) == 0:
            return np.zeros(0)
        m = np.asarray(t["module_index"])[idx] - 1
        return cos_incidence(np.asarray(t["position"], np.float64)[idx],
                             np.asarray(t["direction"], np.float64)[idx], sph[m, :3], sph[m, 3])

    # Hits present on one side only should be grazing (ill-conditioned); a few
    # others may end just beyond a step end or follow an amplified trajectory.
    total = len(common) + len(only_g) + len(only_w)
    nongrazing = 0
    diag = []
    for t, idx, name in ((got, only_g, "got"), (want, only_w, "want")):
        c = cos_of(t, idx)
        nongrazing += int(np.sum(c >= grazing_cos))
        for i, ci in zip(idx[:5], c[:5]):
            diag.append((name, int(np.asarray(t["photon_index"])[i]), round(float(ci), 4),
                         int(np.asarray(t["n_steps"])[i]),
                         round(float(np.asarray(t["dist_travelled"])[i]), 3)))
    assert nongrazing <= max(1, max_nongrazing * total), (
        f"{nongrazing} non-grazing one-sided hits of {total}: {diag}")
    grazing = len(only_g) + len(only_w) - nongrazing
    assert len(common) + grazing >= min_match * total, (len(common), total, diag)

    g = {k: np.asarray(v)[ig] for k, v in got.items() if hasattr(v, "__len__")}
    w = {k: np.asarray(v)[iw] for k, v in want.items() if hasattr(v, "__len__")}
    np.testing.assert_array_equal(g["module_index"], w["module_index"])
    np.testing.assert_array_equal(g["n_steps"], w["n_steps"])
    np.testing.assert_allclose(g["wavelength"], w["wavelength"], rtol=1e-5)
    np.testing.assert_allclose(g["initial_direction"], w["initial_direction"], atol=1e-5)
    ddir = np.linalg.norm(np.asarray(g["direction"], np.float64) -
                          np.asarray(w["direction"], np.float64), axis=1)
    assert np.quantile(ddir, 0.99) <= max(rel, 1e-5) * 10, np.quantile(ddir, 0.99)

    m = np.asarray(w["module_index"]) - 1
    wp = np.asarray(w["position"], np.float64)
    cinc = np.maximum(cos_of(want, iw), 1e-6)
    L = np.asarray(w["dist_travelled"], np.float64) + sph[m, 3]
    # accumulated rounding grows with the path, so the scale is the larger of
    # |position| and the distance travelled
    scale = np.maximum.reduce([np.ones(len(wp)), np.linalg.norm(wp, axis=1),
                               np.asarray(w["dist_travelled"], np.float64)])
    cond = cond_factor * EPS32 * L ** 2 / (2 * sph[m, 3] * cinc)
    dpos = np.linalg.norm(np.asarray(g["position"], np.float64) - wp, axis=1)
    bad = dpos > rel * scale + cond
    assert not np.any(bad), (f"{bad.sum()} hits outside tolerance; worst "
                             f"{dpos[bad][:3]} vs {(rel * scale + cond)[bad][:3]}")
    ddist = np.abs(np.asarray(g["dist_travelled"], np.float64) -
                   np.asarray(w["dist_travelled"], np.float64))
    assert np.all(ddist <= rel * scale + cond), "dist_travelled mismatch"
    wt = np.asarray(w["time"], np.float64)
    dt = np.abs(np.asarray(g["time"], np.float64) - wt)
    v = np.asarray(w["dist_travelled"], np.float64) / np.maximum(wt, 1e-9)
    assert np.all(dt <= rel * np.maximum(1.0, np.abs(wt)) + (rel * scale + cond) /
                  np.maximum(v, 1e-3)), "time mismatch"
    relpos = dpos / scale
    return dict(matched=len(common), only_got=len(only_g), only_want=len(only_w),
                pos_rel_p50=float(np.median(relpos)) if len(relpos) else 0.0,
                pos_rel_p99=float(np.quantile(relpos, 0.99)) if len(relpos) else 0.0,
                pos_abs_max=float(dpos.max()) if len(dpos) else 0.0,
                frac_within_1e5=float(np.mean(relpos <= rel)) if len(relpos) else 1.0)


def oracle_columns(hits):
    return {k: hits[k] for k in hits.dtype.names}


def spheres_of(setup):
    return np.array([[*t.shape.position, t.shape.radius] for t in setup.targets], np.float64)
