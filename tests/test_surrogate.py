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
