"""DOM and generic multi-PMT detection (src/dom.jl, src/generic_multipmt.jl,
src/detection.jl:90-131): the tables, the oracle against literal per-hit
restatements and the defining probabilities, the host API, and the device
kernel against the oracle decision by decision."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
# the reference checkout whose asset tables the committed CSVs are extracted from
REF_ROOT = os.environ.get("PP_REFERENCE_ROOT", "")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pmt_oracle  # noqa: E402


def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True)


def _dom_dict(pp, orientation=None, apply_wl=True):
    m = pp.dom.dom_model(orientation=orientation, apply_wl_acc=apply_wl)
    return dict(poly=np.array(m.poly[:m.n_poly]), polymax=m.polymax,
                zenith_axis=np.array(m.zenith_axis[:]), wl=np.array(m.wl[:m.n_wl]),
                wl_acc=np.array(m.wl_acc[:m.n_wl]), apply_wl=apply_wl)


def _multipmt_dict(pp, target, orientation=None):
    m = pp.generic_multipmt.multipmt_model([target], orientation)
    n = m.n_pmt
    return dict(pmt_dir_module=np.array([m.pmt_dir_module[i][:] for i in range(n)]),
                pmt_dir=np.array([m.pmt_dir[i][:] for i in range(n)]), pmt_area=m.pmt_area,
                qe_wavelength=np.array(m.qe_wavelength[:m.n_qe]), qe=np.array(m.qe[:m.n_qe]))


def test_tables(pp):
    a = pp.dom.load_dom_acceptance()
    assert len(a.poly) == 11 and a.polymax == pytest.approx(0.6301765262123344)
    x = np.linspace(-1, 1, 2001)
    y = a.angular(x)
    assert y.min() > 0 and y.max() == pytest.approx(a.polymax, rel=2e-3)
    assert a.wl[0] == 260 and a.wl[-1] == 680 and np.all(np.diff(a.wl) > 0)
    # effective area / DOM cross-section
    assert a.wl_acc.max() == pytest.approx(0.0114425 / (np.pi * 0.16510 ** 2), rel=1e-12)
    t = pp.make_generic_multipmt_om([1.0, 2.0, 3.0], 0.2, 7)
    assert pp.generic_multipmt.get_pmt_count(t) == 20
    assert t.pmt_area == pytest.approx((0.0762 / 2) ** 2 * np.pi)
    d = pp.generic_multipmt.get_pmt_positions(t)
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-12)
    R = np.array([[0, 0, 1.0], [0, 1, 0], [-1, 0, 0]])
    np.testing.assert_allclose(pp.generic_multipmt.get_pmt_positions(t, R), d @ R.T, atol=1e-12)
    assert t.wl_acceptance(400.0) == pytest.approx(
        np.interp(400.0, *pp.generic_multipmt.load_multipmt_qe()))
    assert t.wl_acceptance(900.0) == 0.0
    f = pp.fibonacci_sphere(50)
    np.testing.assert_allclose(np.linalg.norm(f, axis=1), 1.0, atol=1e-12)
    assert f[0, 1] == 1.0 and f[-1, 1] == -1.0


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "assets")),
                    reason="set PP_REFERENCE_ROOT to a reference checkout with its assets")
def test_tables_extracted_from_reference(tmp_path, monkeypatch):
    """The committed CSVs are what the extraction script makes from the
    reference's assets."""
    sys.path.insert(0, os.path.join(ROOT, "photonpropagation.jl_gb300", "data"))
    import extract_detection_tables as ex
    monkeypatch.setattr(ex, "HERE", str(tmp_path))
    ex.main(REF_ROOT)
    data = os.path.join(ROOT, "photonpropagation.jl_gb300", "data")
    for f in ("dom_angular_acceptance.csv", "dom_wl_acceptance.csv", "multipmt_qe.csv"):
        assert open(tmp_path / f).read() == open(os.path.join(data, f)).read(), f


def test_dom_oracle_rates(pp):
    """Detection rate = E[min(poly(cos z) / polymax, 1)] x E[wl_acc] for
    independent uniforms; the zenith is taken in the module frame."""
    rng = np.random.default_rng(3)
    n = 400_000
    dirs = _unit(rng, n)
    wl = rng.uniform(300, 700, n)
    R = np.array([[1.0, 0, 0], [0, 0, -1], [0, 1, 0]])  # module z axis along detector y... turned
    for orientation in (None, R):
        m = _dom_dict(pp, orientation)
        targets = [dict(position=[0, 0, 0], radius=0.1651, kind="dom", active_area=0.0)]
        pos = 0.1651 * _unit(rng, n)
        ids, qe = pmt_oracle.detect(pos, wl, np.ones(n), targets, dict(dom=m), seed=4,
                                    directions=dirs)
        a = pp.dom.load_dom_acceptance()
        cz = dirs @ (np.eye(3) if orientation is None else R)[:, 2]
        p = np.minimum(a.angular(cz) / a.polymax, 1.0) * a.wavelength(wl)
        assert abs(ids.sum() - p.sum()) < 5 * np.sqrt(p.sum()), (ids.sum(), p.sum())
        assert set(np.unique(ids)) <= {0, 1} and np.all(qe == 1.0)
    # without the wavelength acceptance only the angular test remains
    ids, _ = pmt_oracle.detect(pos, wl, np.ones(n), targets, dict(dom=_dom_dict(pp, None, False)),
                               seed=4, directions=dirs)
    p = np.minimum(a.angular(dirs[:, 2]) / a.polymax, 1.0)
    assert abs(ids.sum() - p.sum()) < 5 * np.sqrt(p.sum())


def _statsbase_scan(w, u):
    """StatsBase 0.34 sample(rng, wv): t = u * sum(w); i = 1, cw = w[1];
    while cw < t and i < n: i += 1, cw += w[i]."""
    t = u * w.sum(dtype=w.dtype)
    i, cw = 0, w[0]
    while cw < t and i < len(w) - 1:
        i += 1
        cw = w.dtype.type(cw + w[i])
    return i + 1


def test_multipmt_oracle_against_literal_restatement(pp):
    """The vectorised oracle = a literal per-hit loop of the reference's steps
    in the same FP32 order; and against FP64 the choice agrees but for
    weights that sum to ~0 (the reference's weights -(rel . p) over PMT axes
    that nearly cancel)."""
    rng = np.random.default_rng(5)
    t = pp.make_generic_multipmt_om([1.0, -2.0, 0.5], 0.2, 3)
    R = np.array([[0.0, -1, 0], [1, 0, 0], [0, 0, 1]])
    m = _multipmt_dict(pp, t, R)
    n = 3000
    rel = _unit(rng, n)
    pos = (np.array(t.shape.position) + 0.2 * rel).astype(np.float32)
    dirs = -rel + 0.3 * _unit(rng, n)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    wl = rng.uniform(290, 720, n)
    targets = [dict(position=t.shape.position, radius=0.2, kind="multipmt", active_area=0.0)]
    ids, qe = pmt_oracle.detect(pos, wl, np.ones(n), targets, dict(multipmt=m), seed=11,
                                directions=dirs)
    rows = np.arange(n, dtype=np.uint64)
    r = pmt_oracle.philox4x32_10(rows, rows >> np.uint64(32), np.full(n, pmt_oracle.PMT_STREAM),
                                 np.zeros(n), 11, 0)
    u1, u2 = pmt_oracle.u01(r[0]), pmt_oracle.u01(r[1])
    f32 = np.float32
    want = np.zeros(n, np.int32)
    agree64 = 0
    qm, qo = m["pmt_dir_module"].astype(f32), m["pmt_dir"].astype(f32)
    d32 = dirs.astype(f32)
    c0 = np.array(t.shape.position, f32)
    for i in range(n):
        proj = f32(0)
        for k in range(20):
            c = f32(f32(f32(d32[i, 0] * qm[k, 0]) + f32(d32[i, 1] * qm[k, 1])) +
                    f32(d32[i, 2] * qm[k, 2]))
            if c > 0:
                proj = f32(proj + c)
        prob = f32(f32(proj * f32(m["pmt_area"])) / f32(f32(f32(3.14159265358979) * f32(0.2)) *
                                                           f32(0.2)))
        if not u1[i] <= prob:
            continue
        rl = ((pos[i] - c0) * f32(f32(1) / f32(0.2))).astype(f32)
        w = np.array([-f32(f32(f32(rl[0] * qo[k, 0]) + f32(rl[1] * qo[k, 1])) +
                           f32(rl[2] * qo[k, 2])) for k in range(20)], f32)
        want[i] = _statsbase_scan(w, u2[i])
        # the reference's own FP64 form
        rl64 = (pos[i].astype(float) - np.array(t.shape.position)) / 0.2
        w64 = -(get := pp.generic_multipmt.get_pmt_positions(t, R)) @ rl64
        del get
        agree64 += _statsbase_scan(w64, float(u2[i])) == want[i]
    np.testing.assert_array_equal(ids, want)
    hit = want > 0
    assert hit.sum() > 200
    assert agree64 / hit.sum() > 0.98
    # hit probability = projected PMT area / cross-section, QE = R6091 / 100
    np.testing.assert_allclose(qe, pmt_oracle.interp0(m["qe_wavelength"], m["qe"], wl),
                               rtol=0, atol=0)


def test_multipmt_hit_probability(pp):
    rng = np.random.default_rng(6)
    t = pp.make_generic_multipmt_om([0.0, 0.0, 0.0], 0.2, 1)
    m = _multipmt_dict(pp, t)
    n = 300_000
    dirs = _unit(rng, n)
    pos = 0.2 * _unit(rng, n)
    targets = [dict(position=[0, 0, 0], radius=0.2, kind="multipmt", active_area=0.0)]
    ids, _ = pmt_oracle.detect(pos, np.full(n, 400.0), np.ones(n), targets, dict(multipmt=m), 2,
                               directions=dirs)
    q = pp.generic_multipmt.get_pmt_positions(t)
    p = np.clip(dirs @ q.T, 0, None).sum(axis=1) * t.pmt_area / (np.pi * 0.2 ** 2)
    assert abs((ids > 0).sum() - p.sum()) < 5 * np.sqrt(p.sum())
    assert ids.max() <= 20


def test_host_api(pp, tmp_path):
    P = pp.detection
    assert P.check_pmt_hit_opening_angle([0, 0, 1.0], [[1.0, 0, 0], [0, 0.6, 0.8]], 0.7) == 2
    assert P.check_pmt_hit_opening_angle([0, 0, 1.0], [[1.0, 0, 0]], 0.7) == 0
    csv = tmp_path / "qe.csv"
    csv.write_text("wavelength,QE,rel_acceptance\n300,10,0.5\n400,30,1.0\n")
    q = P.InterpQuantumEff.from_csv(str(csv))
    assert q(350.0) == pytest.approx(0.2) and q(250.0) == 0.0
    assert P.InterpQuantumEff.from_csv(str(csv), relative=True)(350.0) == pytest.approx(0.75)
    dom = pp.DOM.at([0.0, 0.0, 0.0], 5)
    mp = pp.make_generic_multipmt_om([5.0, 0.0, 0.0], 0.2, 6)
    table = pp.HitTable(wavelength=np.array([350.0, 450.0]), module_id=np.array([6, 6]),
                        total_weight=np.array([2.0, 3.0]))
    P.calc_pe_weight(table, [dom, mp])
    np.testing.assert_allclose(table["qe_weight"], mp.wl_acceptance([350.0, 450.0]))
    np.testing.assert_allclose(table["total_weight"], [2.0, 3.0] * table["qe_weight"])
    with pytest.raises(NotImplementedError):
        P.calc_pe_weight(pp.HitTable(wavelength=np.array([400.0]), module_id=np.array([5]),
                                     total_weight=np.array([1.0])), [dom, mp])
    tg = P.pmt_targets([dom, mp])
    assert (tg[0].kind, tg[1].kind) == (pp._lib.PP_PMT_DOM, pp._lib.PP_PMT_MULTIPMT)
    with pytest.raises(ValueError):
        other = pp.make_generic_multipmt_om([0.0, 5.0, 0.0], 0.2, 7, pmt_diameter=0.05)
        P.detection_models([mp, other])


def _mixed(pp, n, seed):
    """Hits on a DOM, a multi-PMT module, a POM and a homogeneous module."""
    rng = np.random.default_rng(seed)
    targets = [pp.DOM.at([0.0, 0.0, 0.0], 21), pp.make_generic_multipmt_om([8.0, 0.0, 0.0], 0.2, 22),
               pp.POM.at([0.0, 9.0, 1.0], 23),
               pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 12.0], 0.3), 0.05, 24)]
    mi = rng.integers(1, 5, n)
    centres = np.array([t.shape.position for t in targets], float)
    radii = np.array([t.shape.radius for t in targets], float)
    rel = _unit(rng, n)
    pos = centres[mi - 1] + radii[mi - 1, None] * rel
    dirs = -rel + 0.5 * _unit(rng, n)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    wl = rng.uniform(280, 820, n)
    return targets, pos, dirs, wl, mi


def _oracle_targets(pp, targets):
    kinds = {pp.DOM: "dom", pp.SphericalMultiPMTTarget: "multipmt", pp.POM: "pom",
             pp.HomogeneousDetector: "homogeneous"}
    return [dict(position=t.shape.position, radius=t.shape.radius, kind=kinds[type(t)],
                 active_area=getattr(t, "pmt_area", 0.0)) for t in targets]


def _oracle_model(pp, targets, orientation, apply_wl):
    from test_pmt import _model_dict
    m = _model_dict(pp, orientation)
    m["dom"] = _dom_dict(pp, orientation, apply_wl)
    m["multipmt"] = _multipmt_dict(pp, targets[1], orientation)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("apply_wl", [True, False])
def test_device_matches_oracle(pp, gpu_ctx, apply_wl):
    torch = pytest.importorskip("torch")
    n = 400_000
    targets, pos, dirs, wl, mi = _mixed(pp, n, seed=8)
    R = np.array([[0.0, 0, 1], [0, 1, 0], [-1, 0, 0]])
    rec = np.zeros(n, dtype=np.dtype(pp._lib.pp_hit_record))
    rec["position"] = pos.astype(np.float32)
    rec["direction"] = dirs.astype(np.float32)
    rec["wavelength"] = wl.astype(np.float32)
    rec["module_index"] = mi.astype(np.int32)
    d_rec = torch.from_numpy(rec.view(np.uint8)).cuda()
    d_id = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    d_qe = torch.full((n,), -1.0, dtype=torch.float32, device="cuda")
    pp.detection.make_hits_device(d_rec.data_ptr(), n, targets, 77, d_id.data_ptr(),
                                  d_qe.data_ptr(), orientation=R, apply_wl_acc=apply_wl)
    got_id, got_qe = d_id.cpu().numpy(), d_qe.cpu().numpy()
    want_id, want_qe = pmt_oracle.detect(rec["position"], rec["wavelength"], mi,
                                         _oracle_targets(pp, targets),
                                         _oracle_model(pp, targets, R, apply_wl), 77,
                                         directions=rec["direction"])
    for k in range(1, 5):
        sel = mi == k
        agree = (got_id[sel] == want_id[sel]).mean()
        assert agree > 0.9999, (k, agree)
        assert (got_id[sel] > 0).sum() > 200, k
    np.testing.assert_allclose(got_qe, want_qe, rtol=1e-5, atol=1e-7)


@pytest.mark.gpu
def test_make_hits_from_photons_doms_and_multipmt(pp, gpu_ctx):
    """Propagation onto a DOM and a multi-PMT module, then detection through
    the host API: counts agree with the expectation of the hits' detection
    probabilities."""
    medium = pp.CascadiaMediumProperties()
    dom = pp.DOM.at([0.0, 0.0, 5.0], 1)
    mp = pp.make_generic_multipmt_om([0.0, 5.0, 0.0], 0.3, 2)
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 10_000_000)
    setup = pp.PhotonPropSetup([src], [dom, mp], medium,
                               pp.make_cherenkov_spectrum((300.0, 800.0), medium), 3)
    table = pp.propagate_photons(setup)
    assert table.nrow > 5000
    hits = pp.make_hits_from_photons(table, setup, seed=5)
    a = dom.acceptance
    on_dom = table["module_id"] == 1
    p_dom = (np.minimum(a.angular(table["direction"][on_dom][:, 2]) / a.polymax, 1.0) *
             a.wavelength(table["wavelength"][on_dom]))
    got = (hits["module_id"] == 1).sum()
    assert abs(got - p_dom.sum()) < 5 * np.sqrt(p_dom.sum()) + 5, (got, p_dom.sum())
    on_mp = table["module_id"] == 2
    q = pp.generic_multipmt.get_pmt_positions(mp)
    p_mp = np.clip(table["direction"][on_mp] @ q.T, 0, None).sum(axis=1) * mp.pmt_area / (
        np.pi * 0.3 ** 2)
    got = (hits["module_id"] == 2).sum()
    assert abs(got - p_mp.sum()) < 5 * np.sqrt(p_mp.sum()) + 5, (got, p_mp.sum())
    assert set(np.unique(hits["pmt_id"][hits["module_id"] == 1])) == {1}
    assert hits["pmt_id"][hits["module_id"] == 2].max() <= 20
    hits = pp.detection.calc_pe_weight(pp.make_hits_from_photons(
        pp.HitTable({k: v[on_mp] for k, v in table.items()}), setup, seed=5), setup)
    np.testing.assert_allclose(hits["qe_weight"], mp.wl_acceptance(hits["wavelength"]))


def test_multipmt_as_in_the_reference_example(pp):
    """examples/generic_multipmt_om.jl builds the module from Fibonacci points
    with no wavelength acceptance: the device model gets QE 1, calc_pe_weight
    has no QE to apply (the reference would fail calling nothing)."""
    f = pp.fibonacci_sphere(20)
    theta = np.arccos(np.clip(f[:, 2], -1, 1))
    phi = np.arctan2(f[:, 1], f[:, 0])
    t = pp.SphericalMultiPMTTarget(pp.Spherical([0.0, 0.0, 0.0], 0.25), (0.0762 / 2) ** 2 * np.pi,
                                   np.stack([theta, phi]), None, 1)
    np.testing.assert_allclose(pp.generic_multipmt.get_pmt_positions(t), f, atol=1e-12)
    m = pp.generic_multipmt.multipmt_model([t])
    assert m.n_pmt == 20 and (m.qe[0], m.qe[1]) == (1.0, 1.0)
    with pytest.raises(TypeError):
        pp.detection.apply_qe(np.array([400.0]), t)


def test_apply_wl_acceptance(pp):
    rng = np.random.default_rng(9)
    dom = pp.DOM.at([0.0, 0.0, 0.0], 1)
    wl = rng.uniform(250, 700, 200_000)
    keep = pp.apply_wl_acceptance(np.zeros((len(wl), 3)), np.zeros((len(wl), 3)), wl, dom, rng=rng)
    p = dom.acceptance.wavelength(wl)
    assert abs(keep.sum() - p.sum()) < 5 * np.sqrt(p.sum())
    assert not keep[wl > 680].any()
    pom = pp.POM.at([0.0, 0.0, 0.0], 2)
    assert pp.apply_wl_acceptance(np.zeros((5, 3)), np.zeros((5, 3)), [400.0] * 5, pom).all()


@pytest.mark.gpu
def test_check_pmt_hit_host_api(pp, gpu_ctx):
    """check_pmt_hit for one module runs the device kernel: its decisions are
    the oracle's for module index 1 (for a DOM the angular test only)."""
    rng = np.random.default_rng(12)
    n = 100_000
    rel = _unit(rng, n)
    dirs = -rel + 0.4 * _unit(rng, n)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    wl = rng.uniform(300, 700, n)
    for t, kind, model in (
            (pp.make_generic_multipmt_om([1.0, 2.0, 3.0], 0.3, 4), "multipmt", None),
            (pp.DOM.at([1.0, 2.0, 3.0], 5), "dom", None)):
        pos = (np.array(t.shape.position) + t.shape.radius * rel).astype(np.float32)
        got = pp.check_pmt_hit(pos, dirs, wl, t, seed=21)
        m = dict(multipmt=_multipmt_dict(pp, t)) if kind == "multipmt" else \
            dict(dom=_dom_dict(pp, None, apply_wl=False))
        want, _ = pmt_oracle.detect(pos, wl.astype(np.float32), np.ones(n),
                                    [dict(position=t.shape.position, radius=t.shape.radius,
                                          kind=kind, active_area=t.pmt_area)], m, 21,
                                    directions=dirs.astype(np.float32))
        assert (got == want).mean() > 0.9999, kind
        assert (got > 0).sum() > 500, kind
