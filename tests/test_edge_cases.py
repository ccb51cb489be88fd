"""Edge cases of the propagation path: empty and ragged inputs, no targets,
extreme step counts and the largest target list (65535 spheres), device
against the oracle."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from replay import compare, oracle_columns, spheres_of  # noqa: E402

pytestmark = pytest.mark.gpu


def _run(pp, setup, n_steps=15, capacity=None, precise=1):
    ctx = pp.get_context(0)
    old = ctx.get_tuning()
    try:
        ctx.set_tuning(precise_math=precise)
        setup.upload(ctx)
        n = sum(pp.source_photons(s.photons, setup.photon_scaling) for s in setup.sources)
        rc, nh, nsim = ctx.propagate(setup.source_records(), len(setup.sources), setup.seed,
                                     n_steps, setup.photon_scaling,
                                     capacity if capacity is not None else max(n, 1))
        return rc, (ctx.fetch_hits(nh) if rc == 0 else None), nh, nsim
    finally:
        ctx.set_tuning(precise_math=old.precise_math)


def _targets(pp):
    return [pp.HomogeneousDetector(pp.Spherical(p, 1.0), 1.0, i + 1)
            for i, p in enumerate([[0, 0, 6], [5, 0, 3], [-4, 3, 5], [0, -6, 2]])]


def test_zero_photons_and_zero_scaling(pp, gpu_ctx):
    m = pp.CascadiaMediumProperties()
    spec = pp.make_monochromatic_spectrum(450.0)
    s = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 0)], _targets(pp),
                           m, spec, 1)
    rc, cols, nh, nsim = _run(pp, s)
    assert (rc, nh, nsim) == (0, 0, 0)
    s = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 10_000)],
                           _targets(pp), m, spec, 1, photon_scaling=0.0)
    rc, cols, nh, nsim = _run(pp, s)
    assert (rc, nh, nsim) == (0, 0, 0)
    table = pp.propagate_photons(s)
    assert table.nrow == 0


def test_ragged_sources_replay(pp, orc, gpu_ctx):
    """Photon counts that fill no chunk evenly, one launch."""
    m = pp.CascadiaMediumProperties()
    counts = [0, 1, 31, 33, 1000, 4097, 65_537]
    srcs = [pp.PointlikeIsotropicEmitter([0.3 * i, 0.0, 0.0], float(i), c)
            for i, c in enumerate(counts)]
    s = pp.PhotonPropSetup(srcs, _targets(pp), m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 5)
    rc, cols, nh, nsim = _run(pp, s)
    assert rc == 0 and nsim == sum(counts)
    want, sim, _ = orc.Run.from_setup(s).propagate_all()
    assert sim == sum(counts)
    st = compare(cols, oracle_columns(want), spheres_of(s))
    assert st["matched"] > 500, st
    per_src = np.bincount(cols["source_index"], minlength=len(counts))
    assert per_src[0] == 0 and np.all(per_src[4:] > 0)


def test_no_targets(pp, gpu_ctx):
    m = pp.CascadiaMediumProperties()
    s = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 100_000)], [], m,
                           pp.make_monochromatic_spectrum(450.0), 1)
    rc, cols, nh, nsim = _run(pp, s, precise=0)
    assert (rc, nh, nsim) == (0, 0, 100_000)


@pytest.mark.parametrize("n_steps", [1, 200])
def test_extreme_step_counts(pp, orc, gpu_ctx, n_steps):
    m = pp.CascadiaMediumProperties()
    s = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 50_000)],
                           _targets(pp), m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 3)
    rc, cols, nh, nsim = _run(pp, s, n_steps=n_steps)
    assert rc == 0 and nsim == 50_000
    want, sim, _ = orc.Run.from_setup(s, n_steps=n_steps).propagate_all()
    st = compare(cols, oracle_columns(want), spheres_of(s))
    assert st["matched"] > 100, st
    assert cols["n_steps"].max() <= n_steps


def test_largest_target_list(pp, orc, gpu_ctx):
    """65535 spheres (the index limit of a grid item): a 41 x 41 x 39 lattice
    (plus 36 more) of 0.3 m spheres 4 m apart around the source; the culled
    device search agrees with the oracle's loop over all 65535 targets."""
    g = np.arange(-20, 21) * 4.0
    xs, ys, zs = np.meshgrid(g, g, np.arange(-19, 20) * 4.0 + 2.0, indexing="ij")
    pts = np.stack([xs.ravel(), ys.ravel(), zs.ravel()], 1)
    extra = np.stack([np.arange(36) * 4.0 + 100.0, np.zeros(36), np.zeros(36)], 1)
    pts = np.concatenate([pts, extra])[:65535]
    assert len(pts) == 65535
    targets = [pp.HomogeneousDetector(pp.Spherical(list(p), 0.3), 1.0, (i % 65535) + 1)
               for i, p in enumerate(pts)]
    m = pp.CascadiaMediumProperties()
    s = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0.1, 0.2, 0.3], 0.0, 3000)], targets, m,
                           pp.make_monochromatic_spectrum(450.0), 4)
    rc, cols, nh, nsim = _run(pp, s)
    assert rc == 0 and nsim == 3000 and nh > 300
    run = orc.Run.from_setup(s)
    want, sim, _ = run.propagate_all("f32")
    want64, _, _ = run.propagate_all("f64")
    # on a lattice this dense two spheres can be met in one step at grazing
    # incidence, where the FP32 sphere test is ill-conditioned: a photon that
    # both sides record on different spheres or steps must be one where the
    # FP64 oracle differs from the FP32 one too (one-sided hits are left to
    # compare(), which accepts them only at grazing incidence)
    key = lambda t: {int(p): (int(m), int(n)) for p, m, n in  # noqa: E731
                     zip(t["photon_index"], t["module_index"], t["n_steps"])}
    g, w, w64 = key(cols), key(want), key(want64)
    odd = {p for p in set(g) & set(w) if g[p] != w[p]}
    assert len(odd) <= 5, odd
    assert all(w.get(p) != w64.get(p) for p in odd), [(p, g.get(p), w.get(p), w64.get(p))
                                                       for p in odd]
    keep = lambda t: np.isin(t["photon_index"], list(odd), invert=True)  # noqa: E731
    gk = {k: np.asarray(v)[keep(cols)] for k, v in cols.items()}
    wk = want[keep(want)]
    st = compare(gk, oracle_columns(wk), spheres_of(s))
    assert st["matched"] > 300, st
    assert cols["module_index"].max() > 30_000
