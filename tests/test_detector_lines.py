"""DetectorLines, the per-line pre-culled kernel variant
(src/photon_prop_cuda.jl:552-694): its search order and module numbering in
the oracle, the host types, and the device against the oracle photon by
photon."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import replay  # noqa: E402


def _pencil(pp, lines, photons=20_000, seed=4):
    m = pp.CascadiaMediumProperties()
    src = pp.PencilEmitter([0.0, 0.0, 0.0], [1.0, 0.0, 0.0], 0.0, 0.0, photons)
    return pp.PhotonPropSetup([src], lines, m, pp.make_monochromatic_spectrum(450.0), seed)


def test_records_and_validation(pp):
    lines = pp.DetectorLines([
        pp.DetectorLine(2.0, 0.0, 1.0, [pp.Spherical([2.0, 0.0, 50.0], 0.5)]),
        pp.DetectorLine(5.0, 0.0, 1.0, [pp.Spherical([5.0, 0.0, 0.0], 0.5)])])
    recs = pp.targets.to_targets(lines)
    assert pp.targets.record_count(lines) == 4
    assert [recs[i].kind for i in range(4)] == [pp._lib.PP_TARGET_LINE, pp._lib.PP_TARGET_SPHERE,
                                                pp._lib.PP_TARGET_LINE, pp._lib.PP_TARGET_SPHERE]
    assert recs[0].reserved == 1 and recs[2].position[0] == 5.0 and recs[3].radius == 0.5
    with pytest.raises(ValueError):
        pp.DetectorLines([pp.DetectorLine(0, 0, 1, [pp.Spherical([0, 0, 0], 1)]),
                          pp.DetectorLine(0, 0, 1, [])])
    with pytest.raises(TypeError):
        list(lines)  # not iterable, as in the reference
    setup = _pencil(pp, lines)
    assert setup.has_shaped_targets() and setup.n_target_records() == 4
    # propagate_photons maps module ids by iterating the targets: it fails, as the
    # reference's does (src/processing.jl:67); the driver below returns raw indices
    with pytest.raises(TypeError):
        pp.propagate_photons(setup)


def test_oracle_first_crossed_line_ends_the_search(pp, orc):
    """A pencil beam along +x crosses line 1 (x = 2) in 2-D; its only module is
    far above, so no first-step hit is recorded even where the step reaches
    the module of line 2 at x = 5.  After scattering, photons reach line 2's
    module, reported as module index t + N * line = 1 + 1 * 2 = 3."""
    lines = pp.DetectorLines([
        pp.DetectorLine(2.0, 0.0, 1.0, [pp.Spherical([2.0, 0.0, 50.0], 0.5)]),
        pp.DetectorLine(5.0, 0.0, 1.0, [pp.Spherical([5.0, 0.0, 0.0], 0.5)])])
    setup = _pencil(pp, lines, photons=200_000)
    hits, sim, _ = orc.Run.from_setup(setup).propagate_all()
    assert sim == 200_000
    assert len(hits) > 50
    assert set(np.unique(hits["module_index"])) == {3}
    assert np.all(hits["n_steps"] > 1)
    # the same modules as a plain shape list: first-step hits on the x = 5 module
    plain = _pencil(pp, [pp.HomogeneousDetector(pp.Spherical([2.0, 0.0, 50.0], 0.5), 1.0, 1),
                         pp.HomogeneousDetector(pp.Spherical([5.0, 0.0, 0.0], 0.5), 1.0, 2)],
                    photons=200_000)
    ph, _, _ = orc.Run.from_setup(plain).propagate_all()
    assert (ph["n_steps"] == 1).sum() > 1000


def test_oracle_unnormalised_2d_direction(pp, orc):
    """The 2-D line test takes the (x, y) part of the direction unnormalised
    in the unit-vector formula b = a^2 - (|dp|^2 - r^2).  A beam in the yz
    plane aimed through the centre of the module at (0, 3, 0), with in-plane
    component c, crosses the line in that test only when 9 c^2 >= 9 - 0.25:
    at c = 0.6 the line is never crossed (no first-step hits although the
    beam passes through the module; a plain shape list has them), at
    c = 0.995 it is (module index 1 + 1 * 1 = 2)."""
    m = pp.CascadiaMediumProperties()
    spectrum = pp.make_monochromatic_spectrum(450.0)
    module = pp.Spherical([0.0, 3.0, 0.0], 0.5)
    lines = pp.DetectorLines([pp.DetectorLine(0.0, 3.0, 0.5, [module])])

    def first_step_hits(c, targets):
        s = np.sqrt(1 - c * c)
        src = pp.PencilEmitter([0.0, 0.0, -3.0 * s / c], [0.0, c, s], 0.0, 0.0, 50_000)
        hits, _, _ = orc.Run.from_setup(pp.PhotonPropSetup([src], targets, m, spectrum,
                                                           7)).propagate_all()
        return hits[hits["n_steps"] == 1]

    assert len(first_step_hits(0.6, lines)) == 0
    assert len(first_step_hits(0.6, [pp.HomogeneousDetector(module, 1.0, 1)])) > 1000
    steep = first_step_hits(0.995, lines)
    assert len(steep) > 1000
    np.testing.assert_allclose(np.linalg.norm(steep["position"] - [0.0, 3.0, 0.0], axis=1), 0.5,
                               atol=1e-4)
    assert np.all(steep["module_index"] == 2)


def c1_lines(pp, n_lines=20, n_modules=20, seed=1234, line_radius=5.0):
    """Lines of modules r = 0.2159 m.  The reference's 2-D test registers a
    crossing only when |dp|^2 <= r^2 / (1 - c^2) (c = |dir_xy|), so cylinders
    of the module radius let almost no photon reach a module; a 5 m cylinder
    gives the statistics the comparison needs."""
    rng = np.random.default_rng(seed)
    xy = rng.uniform(-60, 60, size=(n_lines, 2))
    z = np.arange(n_modules) * 6.0 - 57.0
    r = 0.2159
    return pp.DetectorLines([pp.DetectorLine(float(x), float(y), line_radius,
                                             [pp.Spherical([float(x), float(y), float(zz)], r)
                                              for zz in z]) for x, y in xy])


@pytest.mark.gpu
@pytest.mark.parametrize("precise", [1, 0])
def test_device_replays_oracle(pp, orc, gpu_ctx, precise):
    lines = c1_lines(pp)
    m = pp.CascadiaMediumProperties()
    src = pp.PointlikeIsotropicEmitter([1.0, -2.0, 0.5], 0.0, 4_000_000)
    setup = pp.PhotonPropSetup([src], lines, m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 9)
    ctx = pp.Context(0)
    ctx.set_tuning(precise_math=precise)
    setup.upload(ctx)
    recs = setup.source_records()
    rc, nh, nsim = ctx.propagate(recs, 1, setup.seed, 15, setup.photon_scaling, 4_000_000)
    got = ctx.fetch_hits(nh)
    ctx.close()
    assert rc == 0
    want, sim, _ = orc.Run.from_setup(setup).propagate_all()
    assert nsim == sim == 4_000_000
    assert got["module_index"].max() <= 20 * 21 and got["module_index"].min() >= 21
    if precise:
        # spheres by reported module index t + N * l, for the conditioning of
        # the ray-sphere formula (grazing hits after long paths)
        n = lines.modules_per_line
        sph = np.zeros((n * (len(lines.lines) + 1), 4))
        for li, line in enumerate(lines.lines, start=1):
            for t, s in enumerate(line.targets, start=1):
                sph[t + n * li - 1] = [*s.position, s.radius]
        stats = replay.compare(got, replay.oracle_columns(want), sph, mode="precise")
        assert stats["matched"] > 2000, stats
    else:
        g = np.bincount(got["module_index"] // 20, minlength=22)
        w = np.bincount(want["module_index"] // 20, minlength=22)
        assert np.all(np.abs(g - w) <= 5 * np.sqrt(np.maximum(w, 1)) + 5), (g, w)


@pytest.mark.gpu
def test_run_photon_prop_no_local_cache_lines(pp, orc, gpu_ctx):
    """The reference-facing driver returns the kernel's raw module index."""
    lines = c1_lines(pp, n_lines=4, n_modules=5)
    m = pp.CascadiaMediumProperties()
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 500_000)
    cols, n_ph_sim = pp.processing.run_photon_prop_no_local_cache(
        [src], lines, m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 3, pp.HitBuffers(500_000))
    assert n_ph_sim == 500_000
    want, _, _ = orc.Run.from_setup(pp.PhotonPropSetup(
        [src], lines, m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 3)).propagate_all()
    assert abs(len(cols["module_index"]) - len(want)) <= 5 * np.sqrt(len(want)) + 5
    assert set(np.unique(cols["module_index"])) <= set(range(6, 5 * 5 + 1))
