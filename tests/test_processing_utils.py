"""Host utilities of src/processing.jl around the propagation: the number of
steps for a cutoff distance, Poisson resampling of weighted hits, PMT noise."""
import numpy as np
import pytest
from scipy import stats


def test_calc_number_of_steps(pp):
    for sca, cut, q in ((30.0, 100.0, 0.9), (25.0, 300.0, 0.9), (50.0, 20.0, 0.5), (10.0, 100.0, 0.99)):
        n = pp.calc_number_of_steps(sca, cut, q)
        assert n >= int(np.ceil(cut / sca))
        # a fraction q of Erlang(n, sca) paths lies beyond the cutoff ...
        assert stats.gamma.sf(cut, n, scale=sca) >= q
        # ... and n is the first such count from ceil(cut / sca)
        if n > int(np.ceil(cut / sca)):
            assert stats.gamma.sf(cut, n - 1, scale=sca) < q
    # Monte Carlo: sums of n exponential steps
    rng = np.random.default_rng(1)
    n = pp.calc_number_of_steps(30.0, 100.0)
    paths = rng.exponential(30.0, size=(200_000, n)).sum(axis=1)
    assert (paths > 100.0).mean() == pytest.approx(stats.gamma.sf(100.0, n, scale=30.0), abs=5e-3)


def test_resample_hits(pp):
    rng = np.random.default_rng(2)
    n = 4000
    hits = pp.HitTable(module_id=rng.integers(1, 4, n), pmt_id=rng.integers(1, 3, n),
                       total_weight=rng.uniform(0.0, 0.02, n), time=np.arange(n, dtype=float))
    counts = {}
    for rep in range(400):
        r = pp.resample_hits(hits, rng=rng)
        # a subset of the rows, each drawn at most once
        assert len(np.unique(r["time"])) == len(r["time"])
        for m in (1, 2, 3):
            for p in (1, 2):
                counts.setdefault((m, p), []).append(((r["module_id"] == m) & (r["pmt_id"] == p)).sum())
    for (m, p), c in counts.items():
        sel = (hits["module_id"] == m) & (hits["pmt_id"] == p)
        mean = hits["total_weight"][sel].sum()
        assert np.mean(c) == pytest.approx(mean, abs=5 * np.sqrt(mean / 400))
    # heavier hits are drawn more often
    big = pp.HitTable(module_id=np.ones(2, int), pmt_id=np.ones(2, int),
                      total_weight=np.array([0.1, 0.9]), time=np.array([0.0, 1.0]))
    picks = np.concatenate([pp.resample_hits(big, replace=True, rng=rng)["time"] for _ in range(3000)])
    assert (picks == 1.0).mean() == pytest.approx(0.9, abs=0.02)


def test_add_pmt_noise(pp):
    rng = np.random.default_rng(3)
    targets = [pp.POM.at([0.0, 0.0, 0.0], 1), pp.POM.at([0.0, 0.0, 10.0], 2)]
    assert pp.get_pmt_count(targets[0]) == 16
    assert pp.get_pmt_count(pp.DOM.at([0.0, 0.0, 0.0], 3)) == 1
    assert pp.get_pmt_count(pp.make_generic_multipmt_om([0.0, 0.0, 0.0], 0.2, 4)) == 20
    total = 0
    reps = 200
    for _ in range(reps):
        hits = [np.array([5.0]) for _ in range(32)]
        pp.add_pmt_noise(hits, targets, noise_rate=5e4, time_window=2e4, rng=rng)
        for h in hits:
            assert np.all(np.diff(h) >= 0) and 5.0 in h
            assert np.all(np.abs(h) <= 1e4)
            total += len(h) - 1
    # mean noise hits per PMT = 5e4 Hz * 2e4 ns * 1e-9 = 1
    assert total / (32 * reps) == pytest.approx(1.0, abs=5 * np.sqrt(1.0 / (32 * reps)))
