"""ExtendedCherenkovEmitterCustomSmear (src/lightyield.jl:725-769,
src/photon_prop_cuda.jl:134-154): one track-smear table per distinct
Beta(a, b), the index in each source record, and the oracle drawing from it."""
import numpy as np
import pytest


def _setup(pp, srcs, seed=3):
    med = pp.CascadiaMediumProperties()
    targets = [pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 3.0], 2.0), 1.0, 1)]
    return pp.PhotonPropSetup(srcs, targets, med, pp.make_cherenkov_spectrum((300.0, 800.0), med),
                              seed)


def test_tables_and_indices(pp):
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    c = pp.ExtendedCherenkovEmitterCustomSmear
    srcs = [pp.ExtendedCherenkovEmitter([0, 0, 0], [0, 0, 1.0], 0.0, 10, lp),
            c([0, 0, 0], [0, 0, 1.0], 0.0, 10, lp, 2.0, 0.5),
            c([0, 0, 0], [0, 0, 1.0], 0.0, 10, lp),  # the defaults share table 0
            c([0, 0, 0], [0, 0, 1.0], 0.0, 10, lp, 2.0, 0.5),
            pp.PointlikeIsotropicEmitter([0, 0, 0], 0.0, 10)]
    setup = _setup(pp, srcs)
    stack = setup.track_table_stack()
    assert stack.shape == (2, len(setup.track_quantiles()))
    np.testing.assert_array_equal(stack[1], pp.track_smear.beta_track_quantiles(2.0, 0.5))
    recs = setup.source_records()
    assert [recs[i].smear_table for i in range(5)] == [0, 1, 0, 1, 0]
    assert recs[1].kind == pp._lib.PP_SRC_EXTENDED_CHERENKOV
    # a track_smear override replaces table 0 only; default-parameter custom sources then
    # get a Beta table of their own
    over = pp.PhotonPropSetup(srcs, setup.targets, setup.medium,
                              pp.make_cherenkov_spectrum((300.0, 800.0), setup.medium), 3,
                              track_smear=np.linspace(-1, 1, 64).astype(np.float32))
    assert over.track_table_stack().shape == (3, 64)
    assert [over.source_records()[i].smear_table for i in range(5)] == [0, 1, 2, 1, 0]


def test_oracle_draws_from_the_source_table(pp, orc):
    """Beta(1e3, 1e-3) puts the track along the axis: every photon starts on
    the Cherenkov cone, cos(angle to the axis) = 1 / n(wavelength); the
    default table spreads the angles."""
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    srcs = [pp.ExtendedCherenkovEmitterCustomSmear([0, 0, 0], [0, 0, 1.0], 0.0, 100_000, lp,
                                                   1e3, 1e-3),
            pp.ExtendedCherenkovEmitter([0, 0, 0], [0, 0, 1.0], 0.0, 100_000, lp)]
    setup = _setup(pp, srcs)
    hits, sim, _ = orc.Run.from_setup(setup).propagate_all()
    assert sim == 200_000
    n = setup.medium.phase_refractive_index(hits["wavelength"])
    cos_axis = hits["initial_direction"][:, 2]
    tight = hits["source_index"] == 0
    assert tight.sum() > 200 and (~tight).sum() > 200
    # (the quantile table resolves the tail of order b of the Beta below 1)
    on_cone = np.abs(cos_axis - 1.0 / n) < 2e-3
    assert on_cone[tight].mean() > 0.98, on_cone[tight].mean()
    assert on_cone[~tight].mean() < 0.3
    assert np.mean(np.abs(cos_axis[~tight] - 1.0 / n[~tight]) > 0.05) > 0.2


def test_particle_constructor(pp):
    m = pp.CascadiaMediumProperties()
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), m)
    P = pp.particles
    p = P.Particle([1, 2, 3], [0, 0, 1], 5.0, 100.0, 0.0, "EMinus")
    e = P.extended_cherenkov_emitter_custom_smear(p, m, spec, 2.5, 0.3,
                                                  rng=np.random.default_rng(1))
    assert isinstance(e, pp.ExtendedCherenkovEmitterCustomSmear)
    assert (e.cherenkov_beta_a, e.cherenkov_beta_b) == (2.5, 0.3)
    ly = P.total_lightyield(p, m, spec)
    assert abs(e.photons - ly) < 6 * np.sqrt(ly)
