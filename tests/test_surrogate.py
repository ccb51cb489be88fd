"""Surrogate tables and pairs: the histogram mode of the MC kernel against the
CPU oracle's hit lists, and the pair sampler / feature map on the CPU."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def test_sample_pairs_distributions(pp):
    s = pp.surrogate
    p = s.sample_pairs(200_000, seed=3)
    assert p.distance.min() >= s.D_MIN and p.distance.max() <= s.D_MAX
    # log-uniform distance: log d uniform on [log 5, log 300]
    u = (np.log(p.distance) - np.log(s.D_MIN)) / (np.log(s.D_MAX) - np.log(s.D_MIN))
    assert abs(u.mean() - 0.5) < 0.005 and abs(u.var() - 1 / 12) < 0.002
    for v in (p.module_dir, p.emitter_dir):
        np.testing.assert_allclose(np.linalg.norm(v, axis=1), 1.0, rtol=1e-12)
        assert np.all(np.abs(v.mean(axis=0)) < 0.01)  # uniform on the sphere
    assert np.all(s.in_training_range(p))


def test_pair_features(pp):
    s = pp.surrogate
    p = s.sample_pairs(1000, seed=4)
    x = s.pair_features(p)
    assert x.shape == (1000, s.N_FEATURES) and x.dtype == np.float32
    ct = np.sum(p.emitter_dir * p.module_dir, axis=1)
    np.testing.assert_allclose(x[:, 1], ct, atol=1e-6)
    np.testing.assert_allclose(x[:, 1] ** 2 + x[:, 2] ** 2, 1.0, atol=1e-5)
    np.testing.assert_allclose(x[:, 3] ** 2 + x[:, 4] ** 2, 1.0, atol=1e-5)
    # a rotation about z changes only the azimuth features
    c, sn = np.cos(0.7), np.sin(0.7)
    R = np.array([[c, -sn, 0], [sn, c, 0], [0, 0, 1.0]])
    q = s.Pairs(p.distance, p.module_dir @ R.T, p.emitter_dir @ R.T, p.spectrum_id)
    y = s.pair_features(q)
    np.testing.assert_allclose(y[:, [0, 1, 2, 7]], x[:, [0, 1, 2, 7]], atol=1e-5)
    out = s.Pairs(np.array([4.0, 301.0, 10.0]), p.module_dir[:3], p.emitter_dir[:3],
                  np.array([0, 0, 1]))
    assert not np.any(s.in_training_range(out))


def test_cascade_records_match_emitter_records(pp):
    s = pp.surrogate
    p = s.sample_pairs(50, seed=6)
    fast = s.cascade_records(p, 123_456)
    slow = s.table_setup(p, 123_456, seed=1).source_records()
    assert bytes(fast) == bytes(slow)


def oracle_histograms(orc, pp, pairs, photons, seed, n_bins):
    """Counts and log-residual-time histograms from the oracle's hit lists,
    binned with the kernel's FP32 arithmetic."""
    s = pp.surrogate
    setup = s.table_setup(pairs, photons, seed)
    hits, sim, _ = orc.Run.from_setup(setup).propagate_all()
    tgeo = s.geometric_time(pairs, setup.medium).astype(np.float32)
    f32 = np.float32
    tres = (hits["time"] - tgeo[hits["source_index"]].astype(np.float64)).astype(f32)
    u = np.log10(np.maximum(tres + f32(s.T_OFFSET), f32(1e-30))).astype(f32)
    inv = f32(n_bins) / (f32(s.LOG_T_HI) - f32(s.LOG_T_LO))
    b = np.clip(np.floor((u - f32(s.LOG_T_LO)) * inv).astype(np.int64), 0, n_bins - 1)
    n = len(pairs)
    counts = np.bincount(hits["source_index"], weights=hits["abs_weight"], minlength=n)
    hist = np.zeros((n, n_bins))
    np.add.at(hist, (hits["source_index"], b), hits["abs_weight"])
    return counts, hist, sim


@pytest.mark.gpu
def test_histogram_tables_match_oracle(pp, orc, gpu_ctx):
    s = pp.surrogate
    rng = np.random.default_rng(8)
    n = 6
    pairs = s.Pairs(rng.uniform(5.0, 8.0, n), s._unit(rng, n), s._unit(rng, n),
                    np.zeros(n, np.int32))
    photons, seed = 300_000, 11
    ctx = pp.get_context(0)
    old = ctx.get_tuning()
    try:
        ctx.set_tuning(precise_math=1)
        counts, hists = s.generate_tables(pairs, photons, seed=seed, ctx=ctx)
    finally:
        ctx.set_tuning(block_threads=old.block_threads, photons_per_thread=old.photons_per_thread,
                       ctas_per_sm=old.ctas_per_sm, precise_math=old.precise_math,
                       cell_size=old.cell_size, grid_in_global=old.grid_in_global)
    want_c, want_h, sim = oracle_histograms(orc, pp, pairs, photons, seed, s.N_BINS)
    assert sim == n * photons
    assert want_c.sum() > 50
    # one grazing hit may differ per source: at most one weight (< 1) apart
    assert np.all(np.abs(counts - want_c) <= 1.0 + 1e-4 * want_c), (counts, want_c)
    np.testing.assert_allclose(hists.sum(axis=1), counts, rtol=1e-4, atol=1e-3)
    l1 = np.abs(hists - want_h).sum()
    assert l1 <= 2.0 + 1e-3 * want_h.sum(), l1


TABLE_PHOTONS = 100_000


@pytest.fixture(scope="module")
def trained(pp, gpu_ctx):
    """A network trained on 1e5 MC tables (1e5 photons each), the way the
    full-size training runs, only smaller."""
    torch = pytest.importorskip("torch")
    s = pp.surrogate
    ctx = pp.get_context(0)
    pairs = s.sample_pairs(100_000, seed=21)
    c, h = s.generate_tables(pairs, TABLE_PHOTONS, seed=21, ctx=ctx, device_out=True)
    x = torch.tensor(s.pair_features(pairs), device="cuda")
    mlp = s.MLP(max_batch=8192, seed=1)
    log = s.train(mlp, x, c, h, steps=2500, batch=8192, lr=1e-3, log_every=500)
    assert np.isfinite(log[-1][1]) and log[-1][1] < log[0][1]
    yield mlp
    mlp.close()


@pytest.mark.gpu
def test_surrogate_gain_over_the_methods_without_it(pp, gpu_ctx, trained):
    """Against a 1e7-photon MC judge, the trained network's counts beat both
    the reference's analytic distance scaling and an MC run of the same cost
    as one training table entry; its time PDFs are close in KS distance; and
    it answers far faster than the MC."""
    import time
    s = pp.surrogate
    ctx = pp.get_context(0)
    ev = s.sample_pairs(300, seed=77)
    judge_ph = 10_000_000
    t0 = time.perf_counter()
    jc, jh = s.generate_tables(ev, judge_ph, seed=5, ctx=ctx)
    mc_rate = len(ev) / (time.perf_counter() - t0)
    lc, _ = s.generate_tables(ev, TABLE_PHOTONS, seed=6, ctx=ctx)
    sur = s.Surrogate(trained, table_photons=TABLE_PHOTONS, ctx=ctx)
    nn_d, pdf_d = sur.infer(ev)
    nn = nn_d.cpu().numpy() * (judge_ph / TABLE_PHOTONS)
    ok = jc >= 400
    assert ok.sum() >= 10
    rel_nn = np.abs(nn - jc)[ok] / jc[ok]
    rel_mc = np.abs(lc * (judge_ph / TABLE_PHOTONS) - jc)[ok] / jc[ok]
    norm = s.fit_analytic_norm(ev.subset(ok), jc[ok], judge_ph)
    rel_an = np.abs(s.analytic_expectation(ev, judge_ph, norm=norm) - jc)[ok] / jc[ok]
    med = {k: float(np.median(v)) for k, v in (("nn", rel_nn), ("mc", rel_mc), ("an", rel_an))}
    assert med["nn"] < 0.08, med
    assert med["nn"] < 0.5 * med["mc"] and med["nn"] < 0.25 * med["an"], med
    ks = s.ks_distance(pdf_d.cpu().numpy()[ok], jh[ok])
    assert np.median(ks) < 0.06, np.median(ks)
    # throughput: one inference launch over 1e5 pairs vs the MC's pairs/s
    import torch
    big = s.sample_pairs(100_000, seed=3)
    x = torch.tensor(s.pair_features(big), device="cuda")
    out = torch.empty(len(big), device="cuda")
    trained.infer(x.data_ptr(), len(big), out.data_ptr())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    trained.infer(x.data_ptr(), len(big), out.data_ptr())
    nn_rate = len(big) / (time.perf_counter() - t0)
    assert nn_rate > 100 * mc_rate, (nn_rate, mc_rate)


@pytest.mark.gpu
def test_surrogate_fallback_and_audit(pp, gpu_ctx, trained):
    s = pp.surrogate
    ctx = pp.get_context(0)
    ev = s.sample_pairs(400, seed=31)
    ev.distance[:5] = [2.0, 3.0, 4.5, 320.0, 500.0]  # outside the training range
    # a loose error bound: this test is about the mechanics, with few judged pairs
    sur = s.Surrogate(trained, table_photons=TABLE_PHOTONS, ctx=ctx, audit_fraction=0.1,
                      max_median_error=0.2)
    r = sur.expectations(ev, photons=1e6, seed=4)
    assert r.audit["n_outside"] == 5 and r.from_mc[:5].all()
    assert 15 <= r.audit["n_audited"] <= 70 and r.from_mc.sum() == 5 + r.audit["n_audited"]
    assert r.audit["passed"], r.audit
    # MC answers (1e7 photons) are scaled to the requested photons
    mc_c, _ = s.generate_tables(ev.subset(np.flatnonzero(r.from_mc)), 10_000_000, seed=4,
                                ctx=ctx)
    np.testing.assert_allclose(r.counts[r.from_mc], mc_c * 0.1, rtol=1e-5)
    seen = r.counts > 0
    np.testing.assert_allclose(r.pdf[seen].sum(axis=1), 1.0, rtol=1e-4)
    assert np.isnan(r.pdf[~seen]).all() and r.from_mc[~seen].all()
    # network answers scale with the requested photons
    r2 = sur.expectations(ev, photons=2e6, seed=4, with_pdf=False)
    nn = ~r.from_mc
    np.testing.assert_allclose(r2.counts[nn], 2 * r.counts[nn], rtol=1e-6)


def test_calibration_groups(pp):
    """Host check of the calibration summary: equal groups by prediction,
    sums, biases and pulls; a calibrated Poisson sample has small pulls, a
    10% overprediction shows in every group."""
    s = pp.surrogate
    rng = np.random.default_rng(4)
    lam = np.exp(rng.uniform(np.log(0.05), np.log(5e4), 5000))
    obs = rng.poisson(lam)
    c = s.calibration(lam, obs)
    assert len(c["groups"]) == 10 and sum(g["n"] for g in c["groups"]) == 5000
    assert all(g["pred_lo"] <= g["pred_hi"] for g in c["groups"])
    assert c["max_abs_pull"] < 4
    bad = s.calibration(1.1 * lam, obs)
    assert all(-0.12 < g["rel_bias"] < -0.07 for g in bad["groups"][3:])


@pytest.mark.gpu
def test_trained_network_cannot_overflow_bf16_activations(pp, gpu_ctx, trained):
    """Over the box of training features, the trained network's hidden
    activations are provably below the largest BF16 of the fused kernel's
    activations, and the audit reports that bound; a network whose weights
    are blown up past it fails the batch's check and is answered by the MC."""
    s = pp.surrogate
    ctx = pp.get_context(0)
    bound = trained.activation_bound()
    assert bound < s.BF16_MAX, bound
    ev = s.sample_pairs(40, seed=17)
    r = s.Surrogate(trained, table_photons=TABLE_PHOTONS, ctx=ctx, audit_fraction=0.0).expectations(
        ev, seed=1, with_pdf=False)
    assert r.audit["activation_bound"] == pytest.approx(bound) and r.audit["passed"]
    blown = s.MLP(max_batch=256, seed=3)
    flat = trained.params()
    W, b = blown.unpack(flat)
    for w in W[:-1]:
        w *= 1e12
    blown.set_params(flat)
    assert blown.activation_bound() >= s.BF16_MAX
    r2 = s.Surrogate(blown, table_photons=TABLE_PHOTONS, ctx=ctx, audit_fraction=0.0,
                     fallback_photons=100_000).expectations(ev, seed=1, with_pdf=False)
    assert not r2.audit["passed"] and r2.from_mc.all()
    blown.close()


@pytest.mark.gpu
def test_surrogate_calibrated_on_all_audited_pairs(pp, gpu_ctx, trained):
    """Every pair audited (not only the bright ones): in each decile of the
    predicted count the summed network prediction agrees with the summed
    1e7-photon MC within 10% or three Poisson standard deviations."""
    s = pp.surrogate
    ctx = pp.get_context(0)
    ev = s.sample_pairs(1500, seed=91)
    sur = s.Surrogate(trained, table_photons=TABLE_PHOTONS, ctx=ctx, audit_fraction=1.0,
                      max_median_error=1.0)
    r = sur.expectations(ev, photons=1e7, seed=8, with_pdf=False)
    cal = r.audit["calibration"]
    assert sum(g["n"] for g in cal["groups"]) == r.audit["n_audited"] > 1400
    for g in cal["groups"]:
        tol = max(0.10, 3.0 / np.sqrt(max(g["sum_pred"], 1e-9)))
        assert abs(g["rel_bias"]) < tol, cal


@pytest.mark.gpu
def test_surrogate_failed_audit_falls_back_to_mc(pp, gpu_ctx):
    """An untrained network fails the audit's error check: the whole batch is
    then answered by the MC."""
    s = pp.surrogate
    ctx = pp.get_context(0)
    mlp = s.MLP(max_batch=256, seed=9)
    ev = s.sample_pairs(60, seed=5)
    ev.distance[:] = np.linspace(5.0, 7.0, 60)
    sur = s.Surrogate(mlp, ctx=ctx, fallback_photons=1_000_000, audit_fraction=0.3,
                      min_audit_hits=50)
    r = sur.expectations(ev, seed=2)
    assert not r.audit["passed"] and r.from_mc.all()
    flagged = s.Surrogate(mlp, ctx=ctx, fallback_photons=1_000_000, audit_fraction=0.3,
                          min_audit_hits=50, on_failure="flag").expectations(ev, seed=2)
    assert not flagged.audit["passed"] and not flagged.from_mc.all()
    mlp.close()


@pytest.mark.gpu
def test_training_checkpoint_resume(pp, gpu_ctx, tmp_path):
    """Parameters and Adam state saved mid-run: resuming from the file
    continues the same trajectory as the uninterrupted run."""
    torch = pytest.importorskip("torch")
    s = pp.surrogate
    rng = np.random.default_rng(3)
    B = 1024
    x = torch.tensor(rng.normal(size=(B, 8)).astype(np.float32), device="cuda")
    c = torch.tensor(rng.poisson(4.0, B).astype(np.float32), device="cuda")
    h = torch.tensor(rng.poisson(0.3, (B, 64)).astype(np.float32), device="cuda")
    a = s.MLP(max_batch=B, seed=2)
    for _ in range(5):
        a.train_step(x.data_ptr(), c.data_ptr(), h.data_ptr(), B, 1e-3)
    path = str(tmp_path / "ckpt.npz")
    a.save(path)
    b = s.MLP.load(path, max_batch=B)
    np.testing.assert_array_equal(a.params(), b.params())
    for net in (a, b):
        for _ in range(5):
            net.train_step(x.data_ptr(), c.data_ptr(), h.data_ptr(), B, 1e-3)
    pa, pb = a.params(), b.params()
    assert np.linalg.norm(pa - pb) <= 1e-3 * np.linalg.norm(pa)
    a.close()
    b.close()


@pytest.mark.gpu
def test_tables_do_not_depend_on_chunking(pp, gpu_ctx):
    """Chunks launched back to back (each chunk's sources uploaded while the
    previous launch may still run) give the tables that separate, synchronised
    runs of the same chunks give."""
    s = pp.surrogate
    ctx = pp.Context(0)
    rng = np.random.default_rng(12)
    n, chunk, photons, seed = 600, 100, 200_000, 3
    pairs = s.Pairs(rng.uniform(5.0, 10.0, n), s._unit(rng, n), s._unit(rng, n),
                    np.zeros(n, np.int32))
    together, _ = s.generate_tables(pairs, photons, seed=seed, ctx=ctx, chunk=chunk)
    apart = np.concatenate([
        s.generate_tables(pairs.subset(slice(lo, lo + chunk)), photons, seed=seed + lo, ctx=ctx,
                          chunk=chunk)[0] for lo in range(0, n, chunk)])
    assert together.sum() > 1000
    np.testing.assert_allclose(together, apart, rtol=1e-4, atol=1e-4)
    ctx.close()


def _fake_tables(pp, n, seed):
    s = pp.surrogate
    rng = np.random.default_rng(seed)
    p = s.sample_pairs(n, seed=seed)
    return p, rng.poisson(3.0, n).astype(np.float32), rng.random((n, s.N_BINS)).astype(np.float32)


def test_table_store_appends_and_reads_back(pp, tmp_path):
    s = pp.surrogate
    st = s.TableStore(str(tmp_path / "tables"))
    assert st.nsims == 0
    a = _fake_tables(pp, 50, 1)
    b = _fake_tables(pp, 30, 2)
    st.append(*a, photons=100_000, seed=1)
    st.append(*b, photons=100_000, seed=2)
    assert s.TableStore(str(tmp_path / "tables")).nsims == 2
    pairs, counts, hists, attrs = st.read()
    np.testing.assert_array_equal(pairs.distance, np.concatenate([a[0].distance, b[0].distance]))
    np.testing.assert_array_equal(pairs.emitter_dir, np.concatenate([a[0].emitter_dir,
                                                                     b[0].emitter_dir]))
    np.testing.assert_array_equal(counts, np.concatenate([a[1], b[1]]))
    np.testing.assert_array_equal(hists, np.concatenate([a[2], b[2]]))
    assert [x["seed"] for x in attrs] == [1, 2]


def test_arrow_tables_round_trip(pp, tmp_path):
    pytest.importorskip("pyarrow")
    s = pp.surrogate
    p, c, h = _fake_tables(pp, 40, 3)
    f = str(tmp_path / "t.arrow")
    s.write_arrow(f, p, c, h, photons=100_000, seed=3)
    q, c2, h2, attrs = s.read_arrow(f)
    np.testing.assert_array_equal(q.distance, p.distance)
    np.testing.assert_array_equal(q.module_dir, p.module_dir)
    np.testing.assert_array_equal(c2, c)
    np.testing.assert_array_equal(h2, h)
    assert attrs == {"photons": 100_000, "seed": 3}
