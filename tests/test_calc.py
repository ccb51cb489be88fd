"""Geometric times and time residuals (src/calc.jl) on the host, and the
device residuals of hit records against them."""
import numpy as np
import pytest


def test_calc_tgeo_cascade(pp):
    m = pp.CascadiaMediumProperties()
    vg = float(m.group_velocity(800.0))
    t = pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 10.0], 0.3), 0.01, 1)
    assert pp.calc_tgeo(10.0, m) == pytest.approx(10.0 / vg, rel=1e-15)
    assert pp.calc_tgeo(10.0, m, target=t) == pytest.approx(9.7 / vg, rel=1e-15)
    assert pp.calc_tgeo(3.0, 0.2) == pytest.approx(15.0)


def test_calc_tgeo_tracks_is_the_cherenkov_path(pp):
    """The closed form equals the time of the direct Cherenkov photon: the
    track reaches the emission point at along - d / tan(theta_c) (at c), the
    photon covers d / sin(theta_c) at c / n_grp, cos(theta_c) = 1 / n_ph."""
    m = pp.CascadiaMediumProperties()
    n_ph = float(m.phase_refractive_index(800.0))
    n_grp = pp.medium.C_VAC_M_NS / float(m.group_velocity(800.0))
    rng = np.random.default_rng(1)
    p0 = rng.normal(size=3) * 10
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    pos = p0 + rng.normal(size=(50, 3)) * 30
    got = pp.calc_tgeo_tracks(p0, d, pos, m)
    along = (pos - p0) @ d
    dist = np.linalg.norm(np.cross(pos - p0, d), axis=1)
    th = np.arccos(1.0 / n_ph)
    c = pp.medium.C_VAC_M_NS
    want = (along - dist / np.tan(th)) / c + dist / np.sin(th) * n_grp / c
    np.testing.assert_allclose(got, want, rtol=1e-12)
    np.testing.assert_allclose(pp.closest_approach_distance(p0, d, pos), dist, rtol=1e-12)
    np.testing.assert_allclose(pp.closest_approach_param(p0, d, pos), along, rtol=1e-12)


def _setup(pp, track):
    m = pp.CascadiaMediumProperties()
    targets = [pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 8.0], 0.3), 0.01, 5),
               pp.HomogeneousDetector(pp.Spherical([6.0, 0.0, 3.0], 0.3), 0.01, 9)]
    if track:
        src = pp.CherenkovTrackEmitter([0.0, 0.0, -20.0], [0.0, 0.0, 1.0], 3.0, 40.0, 10_000_000)
    else:
        src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 3.0, 10_000_000)
    return pp.PhotonPropSetup([src], targets, m, pp.make_cherenkov_spectrum((300.0, 800.0), m), 2)


@pytest.mark.parametrize("track", [False, True])
def test_calc_time_residual_host(pp, track):
    s = _setup(pp, track)
    table = {"time": np.array([100.0, 50.0, 70.0]), "module_id": np.array([5, 9, 5], np.uint16)}
    pp.calc_time_residual(table, s)
    tg = pp.calc.module_tgeo(s)
    np.testing.assert_allclose(table["tres"], [100 - tg[0] - 3, 50 - tg[1] - 3, 70 - tg[0] - 3])


@pytest.mark.gpu
@pytest.mark.parametrize("track", [False, True])
def test_device_time_residuals(pp, gpu_ctx, track):
    torch = pytest.importorskip("torch")
    s = _setup(pp, track)
    table = pp.propagate_photons(s)
    assert table.nrow > 100
    pp.calc_time_residual(table, s)
    rec = pp.detection.records_from_table(table, s.targets)
    rec["time"] = table["time"]
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_tres = torch.empty(table.nrow, dtype=torch.float64, device="cuda")
    pp.calc.time_residuals_device(d_rec.data_ptr(), table.nrow, s, d_tres.data_ptr())
    np.testing.assert_allclose(d_tres.cpu().numpy(), table["tres"], rtol=0, atol=1e-9)
    # nothing arrives earlier than direct light; the track form measures to the
    # module centre, so a hit on the near surface may come r * n_grp / c early
    slack = 0.3 / float(s.medium.group_velocity(800.0)) if track else 0.0
    assert table["tres"].min() > -slack - 0.05
