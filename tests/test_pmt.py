"""Detection step (photon hits -> PMT hits): the POM model and tables, the numpy
oracle pinned to the C oracle's Philox and to the acceptance's defining
property, and the device kernel against the oracle decision by decision."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout whose asset tables the committed CSVs are extracted from
REF_ROOT = os.environ.get("PP_REFERENCE_ROOT", "")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pmt_oracle  # noqa: E402


def _model_dict(pp, orientation=None):
    pom = pp.pom
    t = pom.load_pom_tables()
    return dict(acc_wavelength=t.acc_wavelength, acc_group1=t.acc_group1,
                acc_group2=t.acc_group2, sigma_group1=t.sigma_group1,
                sigma_group2=t.sigma_group2, qe_wavelength=t.qe_wavelength, qe=t.qe,
                pmt_dir=pom.pom_pmt_directions(orientation), pmt_group=pom.POM_PMT_GROUP)


def test_numpy_philox_matches_c_oracle(orc):
    rng = np.random.default_rng(2)
    ctr = rng.integers(0, 2 ** 32, size=(64, 4), dtype=np.uint64)
    for key in ((0, 0), (7, 3), (0xdeadbeef, 0x12345678)):
        got = pmt_oracle.philox4x32_10(ctr[:, 0], ctr[:, 1], ctr[:, 2], ctr[:, 3], *key)
        for i in range(0, 64, 7):
            want = orc.philox(ctr[i], key)
            assert tuple(int(g[i]) for g in got) == tuple(int(w) for w in want)


def test_pom_tables_and_geometry(pp):
    pom = pp.pom
    t = pom.load_pom_tables()
    assert len(t.acc_wavelength) == 26 and t.acc_wavelength[0] == 300 and t.acc_wavelength[-1] == 800
    assert np.all(np.diff(t.acc_wavelength) > 0) and np.all(np.diff(t.qe_wavelength) > 0)
    assert 0 < t.acc_group1.max() < 0.1 and 0 < t.acc_group2.max() < 0.1
    assert 0.1 < t.sigma_group1 < t.sigma_group2 < 0.5
    d = pom.pom_pmt_directions()
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-12)
    # four rings about the module axis (+x after the reference's e_z -> e_x turn)
    polar = np.rad2deg(np.arccos(d[:, 0]))
    for ring, want in ((slice(0, 4), 65.0), (slice(4, 8), 32.5), (slice(8, 12), 115.0),
                       (slice(12, 16), 147.5)):
        np.testing.assert_allclose(polar[ring], want, atol=1e-9)
    assert len({tuple(np.round(v, 9)) for v in d}) == 16
    # orientation turns the PMTs with the module
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1.0]])
    np.testing.assert_allclose(pom.pom_pmt_directions(R), d @ R.T, atol=1e-12)


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "assets")),
                    reason="set PP_REFERENCE_ROOT to a reference checkout with its assets")
def test_pom_tables_extracted_from_reference(pp, tmp_path, monkeypatch):
    """The committed CSVs are what the extraction script makes from the
    reference's assets."""
    sys.path.insert(0, os.path.join(ROOT, "photonpropagation.jl_gb300", "data"))
    import extract_pom_tables as ex
    monkeypatch.setattr(ex, "HERE", str(tmp_path))
    ex.main(REF_ROOT)
    data = os.path.join(ROOT, "photonpropagation.jl_gb300", "data")
    for f in ("pom_pmt_acceptance.csv", "pom_pmt_sigma.csv", "pom_rel_qe.csv"):
        assert open(tmp_path / f).read() == open(os.path.join(data, f)).read(), f


def test_uniform_flux_hits_sum_of_group_acceptances(pp):
    """The reference's normalisation (src/pom.jl:286-292): for photons arriving
    uniformly over the module, the detection probability is
    acc_1(wl) + acc_2(wl)."""
    m = _model_dict(pp)
    rng = np.random.default_rng(4)
    v = rng.normal(size=(400_000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    target = dict(position=[0.0, 0.0, 0.0], radius=0.3)
    for wl in (350.0, 450.0, 600.0):
        p = pmt_oracle.detection_probability(0.3 * v, np.full(len(v), wl), target, m)
        want = (np.interp(wl, m["acc_wavelength"], m["acc_group1"]) +
                np.interp(wl, m["acc_wavelength"], m["acc_group2"]))
        assert p.sum(axis=1).mean() == pytest.approx(want, rel=5e-3)


def test_oracle_sampling_follows_probabilities(pp):
    m = _model_dict(pp)
    rng = np.random.default_rng(5)
    n = 200_000
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    targets = [dict(position=[1.0, 2.0, 3.0], radius=0.3, kind="pom", active_area=0.0)]
    pos = np.array([1.0, 2.0, 3.0]) + 0.3 * v
    wl = rng.uniform(320, 780, n)
    ids, qe = pmt_oracle.detect(pos, wl, np.ones(n), targets, m, seed=9)
    p = pmt_oracle.detection_probability(pos, wl, targets[0], m)
    for k in range(16):
        exp = p[:, k].sum()
        assert abs((ids == k + 1).sum() - exp) < 5 * np.sqrt(exp) + 5, k
    np.testing.assert_allclose(qe, np.interp(wl, m["qe_wavelength"], m["qe"], 0, 0), rtol=1e-5,
                               atol=1e-7)


def _synthetic_hits(pp, n, seed):
    """Hits on three POMs and one homogeneous module, wavelengths past both
    ends of the tables."""
    pom = pp.pom
    rng = np.random.default_rng(seed)
    targets = [pom.POM.at([0.0, 0.0, 0.0], 11), pom.POM.at([10.0, -5.0, 3.0], 12),
               pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 20.0], 0.3), 0.05, 13),
               pom.POM.at([-7.0, 2.0, -4.0], 14)]
    mi = rng.integers(1, 5, n)
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    centres = np.array([t.shape.position for t in targets], float)
    radii = np.array([t.shape.radius for t in targets], float)
    pos = centres[mi - 1] + radii[mi - 1, None] * v
    wl = rng.uniform(280, 820, n)
    return targets, pos, wl, mi


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 123456789012])
def test_device_detection_matches_oracle(pp, gpu_ctx, seed):
    torch = pytest.importorskip("torch")
    pom = pp.pom
    n = 300_000
    targets, pos, wl, mi = _synthetic_hits(pp, n, seed=seed % 1000 + 1)
    rec = np.zeros(n, dtype=np.dtype(pp._lib.pp_hit_record))
    rec["position"] = pos.astype(np.float32)
    rec["wavelength"] = wl.astype(np.float32)
    rec["module_index"] = mi.astype(np.int32)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_id = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_qe = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
    pp.detection.make_hits_device(d_rec.data_ptr(), n, targets, seed, d_id.data_ptr(), d_qe.data_ptr())
    got_id, got_qe = d_id.cpu().numpy(), d_qe.cpu().numpy()
    otargets = [dict(position=t.shape.position, radius=t.shape.radius,
                     kind="pom" if isinstance(t, pom.POM) else "homogeneous",
                     active_area=t.pmt_area) for t in targets]
    want_id, want_qe = pmt_oracle.detect(rec["position"], rec["wavelength"], mi, otargets,
                                         _model_dict(pp), seed)
    # the same uniforms: only decisions within float rounding of a threshold may differ
    assert (got_id == want_id).mean() > 0.9999, (got_id != want_id).sum()
    assert (got_id > 0).sum() > 1000
    np.testing.assert_allclose(got_qe, want_qe, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_make_hits_from_photons_end_to_end(pp, gpu_ctx):
    """Propagation onto POMs, then detection: per-PMT counts agree with the
    expectation of the hit positions' detection probabilities, detection is
    reproducible for a seed, and calc_pe_weight scales the weights by the QE."""
    pom = pp.pom
    medium = pp.CascadiaMediumProperties()
    targets = [pom.POM.at([0.0, 0.0, 6.0], 1), pom.POM.at([0.0, 5.0, 0.0], 2)]
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 10_000_000)
    setup = pp.PhotonPropSetup([src], targets, medium, pp.make_cherenkov_spectrum((300.0, 800.0),
                                                                                  medium), 3)
    table = pp.propagate_photons(setup)
    assert table.nrow > 5000
    hits = pp.detection.make_hits_from_photons(table, setup, seed=5)
    again = pp.detection.make_hits_from_photons(table, setup, seed=5)
    np.testing.assert_array_equal(hits["pmt_id"], again["pmt_id"])
    m = _model_dict(pp)
    for t_ix, t in enumerate(targets):
        rows = table["module_id"] == t.module_id
        p = pmt_oracle.detection_probability(table["position"][rows], table["wavelength"][rows],
                                             dict(position=t.shape.position,
                                                  radius=t.shape.radius), m)
        sel = hits["module_id"] == t.module_id
        for k in range(16):
            exp = p[:, k].sum()
            got = (hits["pmt_id"][sel] == k + 1).sum()
            assert abs(got - exp) < 5 * np.sqrt(exp) + 5, (t_ix, k, got, exp)
    w0 = hits["total_weight"].copy()
    pp.detection.calc_pe_weight(hits, setup)
    qe = np.interp(hits["wavelength"], m["qe_wavelength"], m["qe"], left=0, right=0)
    np.testing.assert_allclose(hits["total_weight"], w0 * qe, rtol=1e-12)
