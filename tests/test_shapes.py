"""Shaped targets (spheres, horizontal rectangles and discs tested in index
order at every step, src/photon_prop_cuda.jl:345-404): the oracle's plane
geometry, and the device against the oracle photon by photon and in counts."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def _pencil_setup(pp, targets, photons=20_000):
    m = pp.CascadiaMediumProperties()
    src = pp.PencilEmitter([0.1, -0.2, 0.0], [0.0, 0.0, 1.0], 0.0, 0.0, photons)
    return pp.PhotonPropSetup([src], targets, m, pp.make_monochromatic_spectrum(450.0), 4)


def test_oracle_pencil_beam_through_a_rectangle(pp, orc):
    """Photons whose first step passes z = 5 hit the rectangle straight above
    the beam at (x0, y0, 5), as target 1; a disc the beam misses stays dark."""
    det = [pp.HomogeneousDetector(pp.Rectangular([0.0, 0.0, 5.0], 1.0, 2.0), 1.0, 7),
           pp.HomogeneousDetector(pp.Circular([3.0, 0.0, 2.0], 0.5), 1.0, 8)]
    setup = _pencil_setup(pp, det)
    assert setup.has_shaped_targets()
    hits, sim, _ = orc.Run.from_setup(setup).propagate_all()
    first = hits[hits["n_steps"] == 1]
    assert len(first) > 100  # photons whose first step reaches z = 5
    np.testing.assert_allclose(first["position"][:, 2], 5.0, atol=1e-5)
    np.testing.assert_allclose(first["position"][:, 0], 0.1, atol=1e-5)
    np.testing.assert_allclose(first["position"][:, 1], -0.2, atol=1e-5)
    assert np.all(first["module_index"] == 1)
    np.testing.assert_allclose(first["dist_travelled"], 5.0, atol=1e-4)
    inside = (np.abs(hits["position"][:, 0]) < 0.5) & (np.abs(hits["position"][:, 1]) < 1.0)
    on_rect = hits["module_index"] == 1
    assert np.all(inside[on_rect])
    on_disc = hits["module_index"] == 2
    if on_disc.any():
        p = hits["position"][on_disc]
        assert np.all((p[:, 0] - 3.0) ** 2 + p[:, 1] ** 2 < 0.25 + 1e-4)
        np.testing.assert_allclose(p[:, 2], 2.0, atol=1e-5)


def _mixed_setup(pp, photons, seed=6):
    m = pp.CascadiaMediumProperties()
    targets = [pp.HomogeneousDetector(pp.Rectangular([0.5, 0.0, 6.0], 3.0, 2.0), 1.0, 1),
               pp.HomogeneousDetector(pp.Circular([0.0, 1.0, -5.0], 1.5), 1.0, 2),
               pp.HomogeneousDetector(pp.Spherical([4.0, 0.0, 0.0], 0.6), 1.0, 3),
               pp.HomogeneousDetector(pp.Circular([0.0, 0.0, 9.0], 4.0), 1.0, 4)]
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, photons)
    return pp.PhotonPropSetup([src], targets, m, pp.make_cherenkov_spectrum((300.0, 800.0), m),
                              seed)


def _run_gpu(pp, setup, precise):
    ctx = pp.Context(0)
    ctx.set_tuning(precise_math=precise)
    setup.upload(ctx)
    recs = setup.source_records()
    n = sum(pp.source_photons(s.photons, setup.photon_scaling) for s in setup.sources)
    rc, nh, nsim = ctx.propagate(recs, len(setup.sources), setup.seed, 15,
                                 setup.photon_scaling, n)
    cols = ctx.fetch_hits(nh)
    ctx.close()
    assert rc == 0
    return cols, nsim


@pytest.mark.gpu
def test_shaped_targets_replay(pp, orc, gpu_ctx):
    setup = _mixed_setup(pp, 300_000)
    got, nsim = _run_gpu(pp, setup, precise=1)
    want, sim, _ = orc.Run.from_setup(setup).propagate_all()
    assert nsim == sim == 300_000
    gk = {int(p): i for i, p in enumerate(got["photon_index"])}
    wk = {int(p): i for i, p in enumerate(want["photon_index"])}
    common = sorted(set(gk) & set(wk))
    union = set(gk) | set(wk)
    assert len(union) > 2000
    assert len(common) >= 0.999 * len(union), (len(common), len(union))
    gi = np.array([gk[p] for p in common])
    wi = np.array([wk[p] for p in common])
    assert np.all(got["module_index"][gi] == want["module_index"][wi])
    assert np.all(got["n_steps"][gi] == want["n_steps"][wi])
    scale = np.maximum(np.abs(want["position"][wi]).max(axis=1), want["dist_travelled"][wi])
    dpos = np.abs(got["position"][gi] - want["position"][wi]).max(axis=1)
    assert np.all(dpos <= 1e-5 * scale + 1e-5), dpos.max()
    np.testing.assert_allclose(got["time"][gi], want["time"][wi], rtol=1e-5)
    for k in (1, 2, 3, 4):
        assert (got["module_index"] == k).sum() > 20, k


@pytest.mark.gpu
def test_shaped_targets_fast_kernel_counts(pp, orc, gpu_ctx):
    setup = _mixed_setup(pp, 1_000_000, seed=8)
    got, _ = _run_gpu(pp, setup, precise=0)
    want, _, _ = orc.Run.from_setup(setup).propagate_all()
    for k in (1, 2, 3, 4):
        g = int((got["module_index"] == k).sum())
        w = int((want["module_index"] == k).sum())
        assert abs(g - w) <= 5 * np.sqrt(max(w, 1)) + 5, (k, g, w)


@pytest.mark.gpu
def test_autotune_with_shaped_targets(pp, gpu_ctx):
    """The autotuner on a context holding a shaped-target list (no grid to
    size) tunes the launch shape only, and the hits do not change."""
    setup = _mixed_setup(pp, 400_000, seed=9)
    ctx = pp.Context(0)
    try:
        setup.upload(ctx)
        recs = setup.source_records()
        ctx.set_sources(recs, len(setup.sources), setup.photon_scaling)
        n = sum(pp.source_photons(s.photons, setup.photon_scaling) for s in setup.sources)
        rc, nh, _ = ctx.propagate(recs, len(setup.sources), setup.seed, 15,
                                  setup.photon_scaling, n)
        before = ctx.fetch_hits(nh)
        t, rate = ctx.autotune(setup.seed, 15, sample_photons=200_000)
        assert rate > 0 and 64 <= t.block_threads <= 1024
        rc2, nh2, _ = ctx.propagate(recs, len(setup.sources), setup.seed, 15,
                                    setup.photon_scaling, n)
        after = ctx.fetch_hits(nh2)
    finally:
        ctx.close()
    assert rc == rc2 == 0 and nh == nh2 > 0
    o1, o2 = np.argsort(before["photon_index"]), np.argsort(after["photon_index"])
    for k in ("position", "module_index", "n_steps"):
        np.testing.assert_array_equal(before[k][o1], after[k][o2], err_msg=k)
