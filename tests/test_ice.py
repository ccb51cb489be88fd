"""Deep ice (HomogenousIceProperties, src/ice_properties.jl): the SPICE
formulas in the two restatements (numpy host, C oracle), the simplified-Liu
phase function, the device tables, and a photon-by-photon replay in ice."""
import ctypes
import os
import sys

import numpy as np
import pytest
from scipy import integrate

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from replay import compare, oracle_columns, spheres_of  # noqa: E402


def test_simplified_liu_inverse_cdf(orc):
    """x = 2 eta^((1-g)/(1+g)) - 1 has the density ~ (1 + x)^(2g/(1-g)): its
    CDF ((1 + x)/2)^((1+g)/(1-g)) returns eta, and its mean is g."""
    L = orc.load()
    for g in (0.5, 0.9, 0.95):
        for eta in (0.01, 0.3, 0.77, 1.0):
            x = L.ppo_sl_cos_f64(g, eta)
            assert ((1 + x) / 2) ** ((1 + g) / (1 - g)) == pytest.approx(eta, rel=1e-12)
            assert L.ppo_sl_cos_f32(g, eta) == pytest.approx(x, abs=2e-6)
        m, _ = integrate.quad(lambda e: L.ppo_sl_cos_f64(g, e), 0.0, 1.0, limit=200)
        assert m == pytest.approx(g, abs=1e-7)


def test_ice_two_restatements_agree(orc, pp):
    L = orc.load()
    med = pp.make_homogenous_clearice_properties()
    m, keep = orc.make_medium(med.oracle_params())
    out = (ctypes.c_double * 4)()
    out32 = (ctypes.c_float * 4)()
    for wl in np.linspace(300, 800, 37):
        L.ppo_medium_eval_f64(ctypes.byref(m), wl, out)
        want = [med.scattering_length(wl), med.group_velocity(wl), med.absorption_length(wl),
                med.phase_refractive_index(wl)]
        np.testing.assert_allclose(list(out), want, rtol=1e-12)
        L.ppo_medium_eval_f32(ctypes.byref(m), wl, out32)
        np.testing.assert_allclose(list(out32), want, rtol=5e-6)


def test_ice_values_and_reference_constants(pp):
    med = pp.make_homogenous_clearice_properties(None, 1.5, 0.5)
    assert med.mean_scattering_angle() == pytest.approx(0.9)
    assert med.hg_weight == pytest.approx(0.45)
    assert med.phase_kind == pp._lib.PP_PHASE_HG_SL
    # b_e(400) = b_dust_400, scattering length = (1 - g) / b_e, scaled
    assert med.scattering_length(400.0) == pytest.approx(0.1 / 0.02331206666666667 * 0.5,
                                                         rel=1e-6)
    # a(400) = a_dust_400 + A exp(-B/400) (1 + 0.01 dT), scaled
    a = 0.006350013 + 6954.09033203125 * np.exp(-6617.754394531250 / 400) * (1 + 0.12115215)
    assert med.absorption_length(400.0) == pytest.approx(1.5 / a, rel=1e-6)
    x = 0.4
    n = 1.55749 - 1.57988 * x + 3.99993 * x ** 2 - 4.68271 * x ** 3 + 2.09354 * x ** 4
    assert med.phase_refractive_index(400.0) == pytest.approx(n, rel=1e-12)
    assert med.group_velocity(400.0) == pytest.approx(
        pp.C_VAC_M_NS / (n * (1.227106 - 0.954648 * x + 1.42568 * x ** 2 - 0.711832 * x ** 3)),
        rel=1e-12)
    # the cascade's radiation length in ice: X0 / rho * 10
    lp = pp.LongitudinalParameterisation.from_energy(1e3, med, "EMinus")
    assert lp.lrad == pytest.approx(39.652 / 0.9216 / 910 * 10, rel=1e-6)
    t = med.tables(300.0, 800.0)
    assert t.phase_kind == pp._lib.PP_PHASE_HG_SL


def _ice_setup(pp, photons=200_000, seed=11):
    med = pp.make_homogenous_clearice_properties()
    targets = [pp.HomogeneousDetector(pp.Spherical(p, 0.5), 1.0, i + 1)
               for i, p in enumerate([[0, 0, 8], [6, 0, 4], [-5, 4, 6], [0, -7, 3], [4, 4, -4]])]
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, photons)
    return pp.PhotonPropSetup([src], targets, med, pp.make_cherenkov_spectrum((300.0, 800.0), med),
                              seed)


def test_oracle_ice_runs_the_sl_branch(orc, pp):
    """Ice photons scatter with HG or simplified Liu: the mixture (45 % HG)
    gives finite hits that differ from pure HG at the same g (the ES branch,
    with es_b = 0, would give NaN), and the photons' first steps agree (the
    choice only enters at the first scatter)."""
    def run(hg_fraction):
        med = pp.make_homogenous_clearice_properties()
        med.hg_weight = hg_fraction
        setup = _ice_setup(pp, photons=50_000)
        setup.medium = med
        hits, sim, _ = orc.Run.from_setup(setup, n_steps=31).propagate_all()
        return hits
    mixed, pure = run(0.45), run(1.0)
    for h in (mixed, pure):
        assert len(h) > 200
        assert np.all(np.isfinite(h["position"])) and np.all(np.isfinite(h["time"]))
    km, kp = set(mixed["photon_index"]), set(pure["photon_index"])
    assert km != kp
    first_m = mixed[mixed["n_steps"] == 1]
    first_p = pure[pure["n_steps"] == 1]
    assert len(first_m) == len(first_p) > 10
    np.testing.assert_array_equal(np.sort(first_m["photon_index"]), np.sort(first_p["photon_index"]))


@pytest.mark.gpu
def test_ice_replay(pp, orc, gpu_ctx):
    setup = _ice_setup(pp)
    ctx = pp.Context(0)
    ctx.set_tuning(precise_math=1)
    setup.upload(ctx)
    rc, nh, nsim = ctx.propagate(setup.source_records(), 1, setup.seed, 31, 1.0, 200_000)
    got = ctx.fetch_hits(nh)
    ctx.close()
    assert rc == 0
    want, sim, _ = orc.Run.from_setup(setup, n_steps=31).propagate_all()
    assert nsim == sim == 200_000
    s = compare(got, oracle_columns(want), spheres_of(setup))
    assert s["matched"] > 1000, s


def test_biased_cherenkov_spectrum(pp):
    """Frank-Tamm times a DOM's wavelength acceptance (the reference's example
    pattern): its CDF at the 0.5 nm knots follows the product, and the device
    table draws no wavelength where the bias is 0 (above 680 nm)."""
    med = pp.make_homogenous_clearice_properties()
    bias = pp.DOM.at([0.0, 0.0, 0.0], 1).acceptance.wavelength
    spec = pp.make_biased_cherenkov_spectrum(bias, (300.0, 800.0), med)
    total = integrate.quad(spec.spectrum, 300, 800, points=[680], limit=400)[0]
    d = spec.spectral_dist
    # (the reference's one 25-point Gauss rule over [300, wl] does not resolve the
    # acceptance table's 10 nm kinks: its CDF is off by up to ~0.3 %, reproduced here)
    for wl in (350.0, 420.0, 500.0, 600.0, 675.0):
        want = integrate.quad(spec.spectrum, 300, wl, limit=400)[0] / total
        assert np.interp(wl, d.wavelengths, d.cdf) == pytest.approx(want, abs=5e-3), wl
    knots = d.device_knots(600)
    assert knots.min() >= 300.0 and knots.max() <= 681.0, knots.max()
    flat = pp.make_biased_cherenkov_spectrum(lambda wl: np.ones_like(np.asarray(wl, float)),
                                             (300.0, 800.0), med)
    np.testing.assert_allclose(flat.spectral_dist.device_knots(600),
                               pp.make_cherenkov_spectrum((300.0, 800.0), med)
                               .spectral_dist.device_knots(600), atol=0.05)
