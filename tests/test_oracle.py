"""The CPU oracle pinned against published known answers (no GPU)."""
import ctypes
import os
import sys

import numpy as np
import pytest
from scipy import integrate, special, stats

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


# Philox4x32-10 known-answer vectors published with Random123 (Salmon et al.).
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(orc, ctr, key, want):
    assert tuple(int(x) for x in orc.philox(ctr, key)) == want


def test_u01_range_and_exactness(orc):
    L = orc.load()
    assert L.ppo_u01(0) == pytest.approx(2.0 ** -24, rel=0)
    assert L.ppo_u01(0xffffffff) == 1.0
    assert L.ppo_u01(0xffffff00) == 1.0
    assert L.ppo_u01(255) == 2.0 ** -24


def test_source_photon_count_fp32_semantics(orc, pp):
    L = orc.load()
    # Int64 * Float32 -> Float32, then the thread split sums to floor().
    for photons, scale in [(100_000, 1.0), (100_000_000, 1.0), (123_456_789, 1.0), (7, 0.53),
                           (2 ** 40 + 1, 1.0), (0, 1.0), (10, 0.0)]:
        want = int(np.floor(np.float32(photons) * np.float32(scale)))
        assert L.ppo_source_photons(photons, scale) == want
        assert pp.source_photons(photons, scale) == want
    # FP32 rounding above 2^24 is kept, as in the reference
    assert L.ppo_source_photons(123_456_789, 1.0) == 123_456_792


def test_hg_inverse_cdf_mean_cosine(orc):
    L = orc.load()
    for g in (0.5, 0.9, 0.95):
        m, _ = integrate.quad(lambda e: L.ppo_hg_cos_f64(g, e), 0.0, 1.0, limit=200)
        assert m == pytest.approx(g, abs=1e-8)
        # the sampled cosine has the HG density: CDF check at a few points
        for eta in (0.1, 0.5, 0.9):
            c = L.ppo_hg_cos_f64(g, eta)
            cdf, _ = integrate.quad(
                lambda x: 0.5 * (1 - g * g) / (1 + g * g - 2 * g * x) ** 1.5, -1, c)
            assert cdf == pytest.approx(eta, abs=1e-8)


def test_es_inverse_cdf(orc):
    L = orc.load()
    b = 0.835
    for eta in (0.01, 0.3, 0.5, 0.77, 0.999):
        c = L.ppo_es_cos_f64(b, eta)
        cdf = ((c + 1) + b / 3 * (c ** 3 + 1)) / (2 + 2 * b / 3)
        assert cdf == pytest.approx(eta, abs=1e-12)
    m1, _ = integrate.quad(lambda e: L.ppo_es_cos_f64(b, e), 0, 1)
    m2, _ = integrate.quad(lambda e: L.ppo_es_cos_f64(b, e) ** 2, 0, 1)
    assert m1 == pytest.approx(0.0, abs=1e-10)
    assert m2 == pytest.approx((2 / 3 + 2 * b / 5) / (2 + 2 * b / 3), abs=1e-10)


def _rot(L, a, b):
    A = (ctypes.c_double * 3)(*a)
    B = (ctypes.c_double * 3)(*b)
    O = (ctypes.c_double * 3)()
    L.ppo_rot_from_ez_f64(A, B, O)
    return np.array(list(O))


def test_rotation_from_ez(orc):
    L = orc.load()
    rng = np.random.default_rng(3)
    for _ in range(200):
        a = rng.normal(size=3)
        a /= np.linalg.norm(a)
        assert np.allclose(_rot(L, a, [0, 0, 1]), a, atol=1e-12)
        b = rng.normal(size=3)
        b /= np.linalg.norm(b)
        c = rng.normal(size=3)
        c /= np.linalg.norm(c)
        rb, rc = _rot(L, a, b), _rot(L, a, c)
        assert np.linalg.norm(rb) == pytest.approx(1.0, abs=1e-12)
        assert rb @ rc == pytest.approx(b @ c, abs=1e-12)  # isometry
        assert np.linalg.det(np.stack([_rot(L, a, e) for e in np.eye(3)])) == pytest.approx(1.0)
    assert np.allclose(_rot(L, [0, 0, 1], [0.1, 0.2, 0.3]), [0.1, 0.2, 0.3])
    assert np.allclose(_rot(L, [0, 0, -1], [0.1, 0.2, 0.3]), [-0.1, -0.2, -0.3])


def test_spectrum_texture_addressing(orc):
    L = orc.load()
    k = np.array([300.0, 400.0, 500.0, 800.0], np.float32)
    kp = k.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    n = len(k)
    # texel i is centred at (i + 0.5) / n; clamp outside
    assert L.ppo_spectrum_sample(kp, n, 0.0001) == 300.0
    assert L.ppo_spectrum_sample(kp, n, 0.125) == 300.0
    assert L.ppo_spectrum_sample(kp, n, 0.25) == pytest.approx(350.0)
    assert L.ppo_spectrum_sample(kp, n, 0.5) == pytest.approx(450.0)
    assert L.ppo_spectrum_sample(kp, n, 1.0) == 800.0


def test_cascadia_medium_two_restatements_agree(orc, pp):
    """C oracle and numpy host restatement of the Cascadia formulas."""
    L = orc.load()
    med = pp.CascadiaMediumProperties()
    m, keep = orc.make_medium(med.oracle_params())
    out = (ctypes.c_double * 4)()
    out32 = (ctypes.c_float * 4)()
    for wl in np.linspace(300, 800, 37):
        L.ppo_medium_eval_f64(ctypes.byref(m), wl, out)
        want = [med.scattering_length(wl), med.group_velocity(wl), med.absorption_length(wl),
                med.phase_refractive_index(wl)]
        np.testing.assert_allclose(list(out), want, rtol=1e-12)
        L.ppo_medium_eval_f32(ctypes.byref(m), wl, out32)
        np.testing.assert_allclose(list(out32), want, rtol=2e-6)


def test_medium_pinned_to_reference_printout(orc, pp):
    """The one medium value the reference itself prints.  examples/axicone.ipynb
    (cell 2) builds the Cascadia medium with g = 0.99 and unit scales and
    prints, at 488 nm, "Absorpion length: 26.775087" and "Scattering length:
    56.86782" (Float32 shortest form).  Neither length depends on g or on the
    pure-water fraction, so CascadiaMediumProperties(0.99, 0.2, 1, 1) must give
    the same two Float32 values in every form that feeds the kernel: the FP64
    host restatement, the oracle's FP32 and FP64 evaluations, and the knot of
    the device table (488 nm falls exactly on a 0.125 nm knot, where the
    kernel's linear interpolation returns the knot itself)."""
    want_abs, want_sca = np.float32(26.775087), np.float32(56.86782)
    med = pp.CascadiaMediumProperties(0.99, 0.2, 1.0, 1.0)
    assert np.float32(med.absorption_length(488.0)) == want_abs
    assert np.float32(med.scattering_length(488.0)) == want_sca
    L = orc.load()
    m, keep = orc.make_medium(med.oracle_params())
    out = (ctypes.c_double * 4)()
    out32 = (ctypes.c_float * 4)()
    L.ppo_medium_eval_f64(ctypes.byref(m), 488.0, out)
    L.ppo_medium_eval_f32(ctypes.byref(m), 488.0, out32)
    assert (np.float32(out[0]), np.float32(out[2])) == (want_sca, want_abs)
    assert (np.float32(out32[0]), np.float32(out32[2])) == (want_sca, want_abs)
    t = med.tables(300.0, 800.0)
    x = (np.float32(488.0) - np.float32(t.wl_min)) * np.float32(1.0 / t.wl_step)
    i = int(x)
    assert float(x) == i  # a knot: the interpolation weight is exactly 0
    assert (t.scattering_length[i], t.absorption_length[i]) == (want_sca, want_abs)


def test_cascadia_values_and_reference_constants(pp):
    med = pp.CascadiaMediumProperties()
    # MixedHGES(0.95, 0.835, 1 - 0.2) and the README's one-argument form
    assert (med.hg_g, med.es_b) == (pytest.approx(0.95), 0.835)
    assert med.hg_weight == pytest.approx(0.8)
    assert pp.CascadiaMediumProperties(0.95).hg_weight == pytest.approx(0.8)
    # absorption table: the reference asset at its 5 nm knots
    wl, al = pp.medium.load_abs_table()
    assert len(wl) == 101 and wl[0] == 300 and wl[-1] == 800
    assert med.absorption_length(450.0) == pytest.approx(27.7, rel=1e-12)
    # Kopelevich: pure water + particles at 7.5e-3 ppm
    x = 550 / 450
    want = 1 / (0.0017 * x ** 4.3 + 1.34 * 7.5e-3 * x ** 1.7 + 0.312 * 7.5e-3 * x ** 0.3)
    assert med.scattering_length(450.0) == pytest.approx(want, rel=1e-12)
    n = med.phase_refractive_index(450.0)
    assert 1.34 < n < 1.36
    assert 0.21 < med.group_velocity(450.0) < 0.22
    # lrad for the cascade parameterisation (about 0.36 m)
    assert 36.08 / med.material_density() * 10 == pytest.approx(0.356, abs=0.005)


def test_medium_tables_interpolation_error(pp):
    med = pp.CascadiaMediumProperties()
    t = med.tables(300.0, 800.0, 0.125)
    wl = np.random.default_rng(0).uniform(300, 800, 5000)
    grid = t.wl_min + t.wl_step * np.arange(t.n_knots)
    for name, fn in (("scattering_length", med.scattering_length),
                     ("group_velocity", med.group_velocity),
                     ("absorption_length", med.absorption_length),
                     ("phase_refractive_index", med.phase_refractive_index)):
        approx = np.interp(wl, grid, getattr(t, name).astype(np.float64))
        np.testing.assert_allclose(approx, fn(wl), rtol=1e-6, err_msg=name)


def test_frank_tamm_knots_vs_independent_quadrature(pp):
    med = pp.CascadiaMediumProperties()
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), med)
    knots = spec.spectral_dist.device_knots(600)
    assert knots.dtype == np.float32 and knots.shape == (600,)
    assert knots[0] == 300.0 and knots[-1] == pytest.approx(800.0)
    assert np.all(np.diff(knots) > 0)
    f = lambda w: pp.frank_tamm(w, med.phase_refractive_index(w))
    tot, _ = integrate.quad(f, 300, 800)
    for i in (60, 200, 300, 450, 590):
        u = i / 599
        c, _ = integrate.quad(f, 300, float(knots[i]))
        assert c / tot == pytest.approx(u, abs=2e-5)


def test_gamma_sampler_moments(orc):
    L = orc.load()
    a, b = 2.0, 0.63
    xs = np.array([L.ppo_gamma_f32(7, 3, p, a, 1 / b, None) for p in range(40000)])
    assert stats.kstest(xs, stats.gamma(a, scale=1 / b).cdf).pvalue > 1e-3
    ys = np.array([L.ppo_gamma_f32(7, 3, p, 0.5, 2.0, None) for p in range(20000)])
    assert stats.kstest(ys, stats.gamma(0.5, scale=2.0).cdf).pvalue > 1e-3


def test_exponential_steps(orc):
    L = orc.load()
    u = (ctypes.c_float * 4)()
    vals = []
    for p in range(20000):
        L.ppo_uniforms(11, 0, p, 1, u)
        vals.append(-np.log(u[0]))
    vals = np.array(vals)
    assert vals.mean() == pytest.approx(1.0, abs=0.03)
    assert stats.kstest(vals, "expon").pvalue > 1e-3


def test_unscattered_hit_fraction(orc, pp):
    """No scattering within reach: the hit fraction is the solid-angle fraction
    (1 - sqrt(1 - r^2/d^2)) / 2."""
    med = pp.SimpleMediumProperties(absorption_length_m=30.0, scattering_length_m=1e7,
                                    phase_refractive_index_value=1.35,
                                    mean_scattering_angle_value=0.9, group_velocity_m_ns=0.2)
    n = 400_000
    setup = pp.workloads.c0_setup(n, medium=med)
    hits, sim, _ = orc.Run.from_setup(setup, n_steps=1).propagate_all()
    p = (1 - np.sqrt(1 - 0.3 ** 2 / 10 ** 2)) / 2
    assert sim == n
    assert stats.binomtest(len(hits), n, p).pvalue > 1e-3
    # unscattered photons enter the near cap: d - r <= dist <= sqrt(d^2 - r^2)
    assert np.all(hits["dist_travelled"] >= 9.7 - 1e-5)
    assert np.all(hits["dist_travelled"] <= np.sqrt(100 - 0.09) + 1e-5)
    assert np.all(hits["n_steps"] == 1)
    np.testing.assert_allclose(hits["time"], hits["dist_travelled"] / 0.2, rtol=1e-6)
    np.testing.assert_allclose(hits["abs_weight"], np.exp(-hits["dist_travelled"] / 30.0),
                               rtol=1e-6)


def test_oracle_thread_count_invariance(orc, pp):
    setup = pp.workloads.c0_setup(50_000)
    r = orc.Run.from_setup(setup)
    a, _ = r.propagate(nthreads=1)
    b, _ = r.propagate(nthreads=4)
    a = np.sort(a, order="photon_index")
    b = np.sort(b, order="photon_index")
    assert len(a) > 0
    np.testing.assert_array_equal(a, b)


def test_photon_ranges_partition_the_run(orc, pp):
    setup = pp.workloads.c0_setup(60_000)
    r = orc.Run.from_setup(setup)
    full, _ = r.propagate()
    parts = [r.propagate(begin=b, end=e)[0] for b, e in ((0, 20_000), (20_000, 45_000),
                                                         (45_000, 60_000))]
    got = np.sort(np.concatenate(parts), order="photon_index")
    np.testing.assert_array_equal(got, np.sort(full, order="photon_index"))


def test_f64_oracle_close_to_f32(orc, pp):
    """FP32 vs FP64 on the same random numbers: the FP32 error of the
    reference's arithmetic, stated (positions within 1e-5 relative except where
    the ray-sphere formula is ill-conditioned at grazing incidence)."""
    from replay import compare, oracle_columns, spheres_of
    setup = pp.workloads.c0_setup(200_000)
    r = orc.Run.from_setup(setup)
    a, _ = r.propagate(precision="f32")
    b, _ = r.propagate(precision="f64")
    st = compare(oracle_columns(a), oracle_columns(b), spheres_of(setup), mode="f32_vs_f64")
    assert st["matched"] > 30
    assert st["frac_within_1e5"] > 0.5
