"""Smaller host functions and types of the reference's API (src/calc.jl,
src/lightyield.jl, src/pom.jl, src/spectrum.jl, src/photon_prop_cuda.jl)."""
import ctypes

import numpy as np
import pytest


def test_shift_particle(pp):
    P = pp.particles
    p = P.Particle([1.0, 2.0, 3.0], [0.0, 0.6, 0.8], 5.0, 100.0, 0.0, "EMinus")
    q = pp.shift_particle(p, 10.0)
    np.testing.assert_allclose(q.position, [1.0, 8.0, 11.0])
    assert q.time == pytest.approx(5.0 + 10.0 / pp.C_VAC_M_NS) and q.energy == 100.0
    r = pp.shift_to_closest_approach(p, [1.0, 8.0, 11.0])
    np.testing.assert_allclose(r.position, [1.0, 8.0, 11.0], atol=1e-12)


def test_time_residual_forms(pp):
    m = pp.CascadiaMediumProperties()
    targets = [pp.HomogeneousDetector(pp.Spherical([0.0, 5.0, 10.0], 0.3), 1.0, 7),
               pp.HomogeneousDetector(pp.Spherical([3.0, 0.0, -4.0], 0.3), 1.0, 9)]
    track = pp.CherenkovTrackEmitter([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 2.0, 50.0, 10)
    casc = pp.PointlikeCherenkovEmitter([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 2.0, 10)
    table = pp.HitTable(time=np.array([60.0, 70.0, 80.0]), module_id=np.array([7, 9, 7]))
    for src, form in ((track, pp.calc_time_residual_tracks), (casc, pp.calc_time_residual_cascades)):
        setup = pp.PhotonPropSetup([src], targets, m, pp.make_monochromatic_spectrum(450.0), 1)
        a = pp.calc_time_residual(dict(table), setup)["tres"]
        b = form(dict(table), setup)["tres"]
        np.testing.assert_allclose(a, b, rtol=1e-12)
    want = 60.0 - pp.calc_tgeo(np.hypot(5.0, 10.0), m, target=targets[0]) - 2.0
    assert b[0] == pytest.approx(want, rel=1e-12)


def test_check_intersection(pp, orc):
    """The host form against the C oracle's ray-sphere routine, and the plane
    shapes' geometry."""
    L = orc.load()
    rng = np.random.default_rng(4)
    s = pp.Spherical([1.0, -2.0, 3.0], 0.7)
    fa = ctypes.c_float * 3
    agree = 0
    for _ in range(2000):
        p = rng.normal(size=3) * 3
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        step = float(rng.exponential(5.0))
        hit, dist = pp.check_intersection(s, p, d, step)
        out = ctypes.c_float()
        ohit = L.ppo_intersect_sphere_f32(fa(*s.position), ctypes.c_float(0.7 * 0.7), fa(*p),
                                          fa(*d), ctypes.c_float(step), ctypes.byref(out))
        agree += bool(hit) == bool(ohit) and (not hit or abs(dist - out.value) < 1e-5)
    assert agree == 2000
    r = pp.Rectangular([0.0, 0.0, 5.0], 2.0, 1.0)
    assert pp.check_intersection(r, [0.5, 0.2, 0.0], [0, 0, 1.0], 6.0) == (True, 5.0)
    assert pp.check_intersection(r, [1.5, 0.2, 0.0], [0, 0, 1.0], 6.0)[0] is False
    assert pp.check_intersection(r, [0.5, 0.2, 0.0], [0, 0, 1.0], 4.0)[0] is False
    c = pp.Circular([0.0, 0.0, -3.0], 0.5)
    assert pp.check_intersection(c, [0.3, 0.3, 0.0], [0, 0, -1.0], 5.0) == (True, 3.0)
    assert pp.check_intersection(c, [0.4, 0.4, 0.0], [0, 0, -1.0], 5.0)[0] is False


def test_lightyield_parameter_types(pp):
    base = pp.get_longitudinal_params("EMinus")
    assert (base.alpha, base.beta, base.b) == (2.01849, 1.45469, 0.63207)
    a, b = pp.get_longitudinal_params("HadronShower", 1e3)
    assert a == pytest.approx(1.58357 + 0.96448 * 3) and b == 0.33833
    m = pp.CascadiaMediumProperties()
    lp = pp.LongitudinalParameterisation.from_energy(1e3, m, "HadronShower")
    assert lp.a == pytest.approx(a) and lp.b == pytest.approx(b)
    t = pp.CherenkovTrackLengthParameters(*pp.particles.TRACK_LENGTH_PARAMETERS["Gamma"])
    assert t.alpha == pytest.approx(5.3208540905)
    assert pp.FastLightsabreMuonEmitter is pp.particles.fast_lightsabre_muon_emitter
    assert issubclass(pp.ExtendedCherenkovEmitter, pp.CherenkovEmitter)


def test_spectrum_pom_and_hit_rows(pp):
    m = pp.CascadiaMediumProperties()
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), m)
    np.testing.assert_array_equal(pp.make_cuda_spectral_dist(spec.spectral_dist, (300, 800), 600),
                                  spec.spectral_dist.device_knots(600))
    mono = pp.make_monochromatic_spectrum(450.0).spectral_dist
    assert pp.make_cuda_spectral_dist(mono) is mono
    assert [pp.get_pom_pmt_group(i) for i in (1, 4, 5, 8, 9, 13, 16)] == [1, 1, 2, 2, 1, 2, 2]
    with pytest.raises(NotImplementedError):
        pp.POMRelativeAcceptance()
    assert isinstance(pp.pom.load_pom_tables(), pp.POMAcceptance)
    t = pp.HitTable(position=np.zeros((2, 3)), direction=np.ones((2, 3)),
                    initial_direction=np.ones((2, 3)), wavelength=np.array([400.0, 500.0]),
                    time=np.array([1.0, 2.0]), dist_travelled=np.array([3.0, 4.0]),
                    module_id=np.array([5, 6]), n_steps=np.array([1, 2]))
    rows = list(t.rows())
    assert len(rows) == 2 and isinstance(rows[1], pp.PhotonHit)
    assert (rows[1].wavelength, rows[1].module_id, rows[1].n_steps) == (500.0, 6, 2)


def test_output_tables_and_events(pp, tmp_path):
    """Hit lists <-> hit tables round trip (with PMT noise added), module and
    source tables, and save_event / read_event."""
    rng = np.random.default_rng(3)
    targets = [pp.POM.at([0.0, 0.0, 0.0], 4), pp.POM.at([0.0, 0.0, 20.0], 9)]
    hits = [np.sort(rng.uniform(0, 100, rng.integers(0, 4))) for _ in range(32)]
    pp.add_pmt_noise(hits, targets, noise_rate=1e5, time_window=1e3, rng=rng)
    table = pp.hit_list_to_dataframe(hits, targets)
    assert len(table["time"]) == sum(len(h) for h in hits)
    back = pp.dataframe_to_hit_list(table, targets)
    for a, b in zip(back, hits):
        np.testing.assert_array_equal(np.sort(a), np.sort(b))
    assert set(np.unique(table["module_id"])) <= {4, 9} and table["pmt_id"].max() <= 16
    # only the second module (target_mask)
    part = pp.hit_list_to_dataframe(hits[16:], targets, [False, True])
    assert set(np.unique(part["module_id"])) <= {9}
    mods = pp.targets_to_dataframe(targets)
    assert len(mods["pmt_id"]) == 32 and mods["module_z"][-1] == 20.0
    P = pp.particles
    p = P.Particle([1.0, 2.0, 3.0], [0.0, 0.0, 1.0], 4.0, 1e3, 0.0, "EMinus")
    info = pp.event_info_to_dataframe(p)
    assert info["energy"][0] == 1e3 and info["z"][0] == 3.0
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    srcs = [pp.ExtendedCherenkovEmitter([1.0, 2.0, 3.0], [0.0, 0.0, 1.0], 4.0, 1234, lp)]
    pp.save_event(str(tmp_path), dict(event_id=7, hits=table, sources=srcs))
    ev = pp.read_event(str(tmp_path), 7)
    np.testing.assert_array_equal(ev["hits"]["time"], table["time"])
    assert ev["sources"]["ExtendedCherenkovEmitter"]["n_photons"][0] == 1234
