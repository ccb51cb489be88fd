"""Particles and light yields (src/lightyield.jl) and the particle -> hits
pipeline (propagate_particles, src/processing.jl:209-240)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def medium_spectrum(pp):
    m = pp.CascadiaMediumProperties()
    return m, pp.make_cherenkov_spectrum((300.0, 800.0), m)


def test_cascade_track_length_and_yield(pp, medium_spectrum):
    m, spec = medium_spectrum
    P = pp.particles
    assert P.cascade_cherenkov_track_length(1.0, "EMinus") == pytest.approx(5.3207078881)
    assert P.cascade_cherenkov_track_length(1e3, "HadronShower") == pytest.approx(
        3.3355182722 * 1e3 ** 1.03662217)
    p = P.Particle([0, 0, 0], [0, 0, 1], 0.0, 1e4, 0.0, "EMinus")
    assert P.particle_shape(p) == "Cascade"
    assert P.total_lightyield(p, m, spec) == pytest.approx(
        spec.spectral_dist.normalization * 5.3207078881 * 1e4 ** 1.00000211, rel=1e-12)


def test_track_yield_integral(pp, medium_spectrum):
    m, spec = medium_spectrum
    P = pp.particles
    p = P.Particle([0, 0, 0], [0, 0, 1], 0.0, 1e3, 250.0, "MuMinus")
    assert P.particle_shape(p) == "Track"
    wl = np.linspace(300, 800, 200_001)
    f = spec.spectrum(wl) * (1 + P.rel_additional_track_length(m.phase_refractive_index(wl), 1e3))
    want = np.trapezoid(f, wl) * 250.0
    assert P.total_lightyield(p, m, spec) == pytest.approx(want, rel=1e-6)
    # the tabulated point at n = 1.33 (lambda 0.1880, kappa 0.0206) within the interpolation
    assert P.rel_additional_track_length(1.33, 1.0) == pytest.approx(0.1880, abs=2e-4)


def test_longitudinal_profile_and_angular_distribution(pp, medium_spectrum):
    m, _ = medium_spectrum
    P = pp.particles
    lp = pp.LongitudinalParameterisation.from_energy(1e3, m, "EMinus")
    z = np.linspace(0, 60, 600_001)
    # a density in shower depth counted in radiation lengths, t = z / lrad
    assert np.trapezoid(P.longitudinal_profile(z[1:], lp), z[1:] / lp.lrad) == pytest.approx(
        1.0, abs=1e-4)
    frac = P.fractional_contrib_long(np.linspace(0, 30, 31), lp)
    assert frac[0] == 0 and frac.sum() == pytest.approx(1.0, rel=1e-12)
    assert P.integral_long_profile(0.0, 2.0, lp) == pytest.approx(
        np.trapezoid(P.longitudinal_profile(z[1:20001], lp), z[1:20001] / lp.lrad), abs=1e-4)
    x = np.linspace(-1, 1, 2_000_001)
    dense = np.trapezoid(P.cherenkov_ang_dist(x, 1.34), x)
    assert P.cherenkov_ang_dist_int_quad(1.34) == pytest.approx(dense, rel=1e-5)
    # the reference's closed form: exact away from the peak; across it, off by
    # 2 (L(cc - 1e-5) - K), L the lower branch and K = a Gamma(1/c) (-b)^(-1/c) / c
    from scipy import special
    a, b, c, d = P.STD_ANG_DIST_PARS
    for n in (1.1, 1.3, 1.34, 1.5):
        cc = 1 / n
        assert P.cherenkov_ang_dist_int_analytic(n, 0.2, 0.6 if n > 1.3 else 0.55) == \
            pytest.approx(P.cherenkov_ang_dist_int_quad(n, 0.2, 0.6 if n > 1.3 else 0.55),
                          rel=1e-9)
        zz = -b * 1e-5 ** c
        L = d * (cc - 1e-5) + a * 1e-5 * special.gammaincc(1 / c, zz) * special.gamma(1 / c) \
            * zz ** (-1 / c) / c
        K = a * special.gamma(1 / c) * (-b) ** (-1 / c) / c
        assert P.cherenkov_ang_dist_int_analytic(n) - P.cherenkov_ang_dist_int_quad(n) == \
            pytest.approx(2 * (L - K), abs=1e-9)
    # the exported function interpolates the closed form on n = 1.1:0.01:1.5
    assert P.cherenkov_ang_dist_int(1.34) == pytest.approx(
        P.cherenkov_ang_dist_int_analytic(1.34), rel=1e-12)
    mid = 0.5 * (P.cherenkov_ang_dist_int_analytic(1.34) + P.cherenkov_ang_dist_int_analytic(1.35))
    assert P.cherenkov_ang_dist_int(1.345) == pytest.approx(mid, rel=1e-12)
    with pytest.raises(ValueError):
        P.cherenkov_ang_dist_int(1.6)


def test_emitters_from_particles(pp, medium_spectrum):
    m, spec = medium_spectrum
    P = pp.particles
    rng = np.random.default_rng(1)
    c = P.Particle([1, 2, 3], [0, 0, 1], 5.0, 100.0, 0.0, "EMinus")
    ly = P.total_lightyield(c, m, spec)
    n = [P.extended_cherenkov_emitter(c, m, spec, rng=rng).photons for _ in range(200)]
    assert abs(np.mean(n) - ly) < 5 * np.sqrt(ly / 200)
    e = P.extended_cherenkov_emitter(c, m, spec, oversample=2.0, rng=rng)
    assert isinstance(e, pp.ExtendedCherenkovEmitter) and e.time == 5.0
    assert abs(e.photons - 2 * ly) < 6 * np.sqrt(2 * ly)
    mu = P.Particle([0, 0, 0], [1, 0, 0], 0.0, 1e4, 100.0, "MuMinus")
    t = P.fast_lightsabre_muon_emitter(mu, m, spec, rng=rng)
    le = np.log10(1e4)
    stoch = 10 ** sum(cf * le ** i for i, cf in enumerate(P.FAST_LIGHTSABRE_COEFFS)) * 100.0
    want = P.total_lightyield(mu, m, spec) + stoch
    assert isinstance(t, pp.CherenkovTrackEmitter) and t.length == 100.0
    assert abs(t.photons - want) < 6 * np.sqrt(want)
    with pytest.raises(ValueError):
        P.fast_lightsabre_muon_emitter(P.Particle([0, 0, 0], [1, 0, 0], 0, 1.0, 1.0, "MuMinus"),
                                       m, spec)


def test_split_and_rescale(pp):
    P = pp.particles
    s = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 1.0, 1003)
    parts = P.split_source(s, 4)
    assert [x.photons for x in parts] == [250, 250, 250, 253]
    assert all(x.position == s.position and x.time == 1.0 for x in parts)
    assert P.rescale_source(s, 1.5).photons == 1505
    with pytest.raises(ValueError):
        P.split_source(pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 3), 4)


@pytest.mark.gpu
def test_propagate_particles_pipeline(pp, gpu_ctx):
    P = pp.particles
    m = pp.CascadiaMediumProperties()
    targets = [pp.POM.at([0.0, 0.0, 10.0], 1), pp.POM.at([0.0, 8.0, 4.0], 2)]
    parts = [P.Particle([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 3e3, 0.0, "EMinus")]
    hits = P.propagate_particles(parts, targets, 3, m, rng=np.random.default_rng(2))
    assert hits is not None and hits.nrow > 50
    for col in ("pmt_id", "tres", "qe_weight", "total_weight"):
        assert col in hits
    assert hits["pmt_id"].min() >= 1 and hits["pmt_id"].max() <= 16
    # tres = time - tgeo(module) - t0, tgeo from the cascade vertex
    tg = {t.module_id: pp.calc_tgeo(np.linalg.norm(t.shape.position), m, target=t)
          for t in targets}
    tgeo = np.array([tg[int(k)] for k in hits["module_id"]])
    np.testing.assert_allclose(hits["tres"], hits["time"] - tgeo, atol=1e-9)
    # causality: light leaves the axis at depth s >= 0 at time s / c (the particle
    # outruns the light, so residuals below zero are physical) and travels at most
    # at the largest group velocity of the spectrum
    # (the minimum over s of s / c + |p - s e_z| / v sits where z - s = rho beta / sqrt(1 - beta^2),
    # beta = v / c, clamped to s >= 0)
    c = pp.medium.C_VAC_M_NS
    v_max = max(float(m.group_velocity(wl)) for wl in np.linspace(300, 800, 501))
    beta = v_max / c
    pos = np.asarray(hits["position"], np.float64)
    rho = np.hypot(pos[:, 0], pos[:, 1])
    s = np.maximum(pos[:, 2] - rho * beta / np.sqrt(1 - beta ** 2), 0.0)
    t_min = s / c + np.sqrt(rho ** 2 + (pos[:, 2] - s) ** 2) / v_max
    assert np.all(hits["time"] >= t_min - 1e-3), (hits["time"] - t_min).min()
    assert hits["tres"].min() < -1.0  # the extended emission is visible
