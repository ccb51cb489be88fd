"""Statistical parity of the benchmarked (fast-math) kernel with the oracle.

The fast kernel's SFU approximations move trajectories by ~1e-3 of the path,
so photon-by-photon replay can only be loose for it; these tests compare the
distributions instead, GPU against the FP32 oracle on independent random
streams (fixed seeds):

* per-module hit counts at detector scale (C1's 400 modules), two-sample
  Poisson chi-square, modules with few expected hits pooled;
* arrival-time, wavelength and path-length distributions, two-sample KS at
  p > 0.01;
* the README example (C0): the arrival-time histogram in 1 ns bins on
  0-500 ns, two-sample chi-square, plus the module's hit count.

This is the reference's own validation pattern -- hit counts compared within
their Poisson intervals (examples/validation.jl:294-295,371-379) -- applied to
the GPU path against the oracle.  All GPU calls go through the C ABI."""
import os
import sys

import numpy as np
import pytest
from scipy import stats

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_gpu_parity import gpu_run  # noqa: E402

P_MIN = 0.01


def two_sample_poisson_chi2(a, b, min_count=10):
    """Chi-square of two Poisson count vectors with equal exposure: under the
    hypothesis of equal means, (a_i - b_i)^2 / (a_i + b_i) summed over bins is
    chi-square with one degree of freedom per bin.  Bins with a_i + b_i below
    min_count are pooled into one.  Returns (chi2, dof, p)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    big = (a + b) >= min_count
    A = np.append(a[big], a[~big].sum())
    B = np.append(b[big], b[~big].sum())
    keep = (A + B) > 0
    A, B = A[keep], B[keep]
    chi2 = float(np.sum((A - B) ** 2 / (A + B)))
    dof = int(A.shape[0])
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def test_two_sample_chi2_helper():
    """The helper's p-value is uniform-ish under the null and small under a
    shifted alternative (host-side check of the statistic itself)."""
    rng = np.random.default_rng(3)
    lam = rng.uniform(2, 200, 60)
    ps = [two_sample_poisson_chi2(rng.poisson(lam), rng.poisson(lam))[2] for _ in range(400)]
    assert 0.35 < np.mean(ps) < 0.65
    assert np.mean(np.array(ps) < 0.05) < 0.1
    assert two_sample_poisson_chi2(rng.poisson(lam), rng.poisson(lam * 1.2))[2] < 1e-3


def _sources_inside_detector(pp, n_sources, photons, rng_seed=77):
    """Isotropic point sources 2-8 m from randomly chosen modules of the C1
    detector, so that many modules collect enough hits for a per-module test."""
    targets, _ = pp.workloads.detector_400()
    rng = np.random.default_rng(rng_seed)
    srcs = []
    for _ in range(n_sources):
        t = targets[rng.integers(len(targets))].shape.position
        v = rng.normal(size=3)
        v *= rng.uniform(2.0, 8.0) / np.linalg.norm(v)
        srcs.append(pp.PointlikeIsotropicEmitter(list(np.asarray(t) + v), 0.0, photons))
    return srcs, targets


def _c1_inside_setup(pp, seed, n_sources=16, photons=500_000):
    srcs, targets = _sources_inside_detector(pp, n_sources, photons)
    medium = pp.CascadiaMediumProperties(0.95, 0.2, 1.0, 1.0)
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), medium)
    return pp.PhotonPropSetup(srcs, targets, medium, spec, seed)


@pytest.mark.gpu
def test_c1_per_module_counts_time_and_wavelength(pp, orc, gpu_ctx):
    """400 modules, Frank-Tamm spectrum, sources inside the array:
    per-module hit counts agree within Poisson (chi-square p > 0.01), and the
    arrival-time, wavelength and path-length distributions pass KS at
    p > 0.01."""
    setup_g = _c1_inside_setup(pp, seed=31)
    setup_o = _c1_inside_setup(pp, seed=32)
    rc, cols, nh, nsim = gpu_run(pp, setup_g)
    assert rc == 0 and nsim == 16 * 500_000
    want, sim_o, _ = orc.Run.from_setup(setup_o).propagate_all()
    assert sim_o == nsim
    n_mod = len(setup_g.targets)
    g = np.bincount(cols["module_index"] - 1, minlength=n_mod)
    o = np.bincount(want["module_index"] - 1, minlength=n_mod)
    assert g.sum() > 5000 and (g + o >= 10).sum() >= 30, (g.sum(), (g + o >= 10).sum())
    chi2, dof, p = two_sample_poisson_chi2(g, o)
    assert p > P_MIN, (chi2, dof, p)
    # arrival times relative to each source's emission (all sources at t = 0)
    assert stats.ks_2samp(cols["time"], want["time"]).pvalue > P_MIN
    assert stats.ks_2samp(cols["wavelength"], want["wavelength"]).pvalue > P_MIN
    assert stats.ks_2samp(cols["dist_travelled"], want["dist_travelled"]).pvalue > P_MIN


@pytest.mark.gpu
def test_c1_single_source_counts_and_time(pp, orc, gpu_ctx):
    """The C1 configuration itself (one isotropic point inside the hull, 2e7
    photons): the total count within Poisson, per-module counts by chi-square
    and the arrival-time distribution by KS."""
    photons = 20_000_000
    setup_g = pp.workloads.c1_setup(photons=photons, seed=41)
    setup_g.seed = 43  # the source position follows the workload seed, the stream .seed
    setup_o = pp.workloads.c1_setup(photons=photons, seed=41)
    setup_o.seed = 44
    rc, cols, nh, nsim = gpu_run(pp, setup_g)
    assert rc == 0 and nsim == photons
    want, sim_o, _ = orc.Run.from_setup(setup_o).propagate_all()
    n_mod = len(setup_g.targets)
    g = np.bincount(cols["module_index"] - 1, minlength=n_mod)
    o = np.bincount(want["module_index"] - 1, minlength=n_mod)
    assert abs(g.sum() - o.sum()) / np.sqrt(g.sum() + o.sum()) < 4
    chi2, dof, p = two_sample_poisson_chi2(g, o)
    assert p > P_MIN, (chi2, dof, p)
    assert stats.ks_2samp(cols["time"], want["time"]).pvalue > P_MIN


@pytest.mark.gpu
def test_fast_kernel_hit_rate_unbiased(pp, orc, gpu_ctx):
    """The fast kernel against the FP64 oracle on the same random streams at C1
    (1.5e7 photons): the photons that hit in only one of the two are as many
    one way as the other (sign test, 3 sigma).

    The reference's sphere test b = a^2 - (|p - c|^2 - r^2) assumes a unit
    direction; a norm error e shifts b by 2 e a^2, at 100 m from a module
    comparable to r^2.  The fast kernel's SFU sine, cosine and square root
    leave norms ~1e-6 off 1, which cost ~3% of the C1 hits before it
    renormalised its directions; FP32 rounding of the reference's own
    arithmetic (the oracle's FP32 build, the replay kernel) drifts the other
    way and gains ~0.7% against FP64.  Paired counts see both; chi-square
    tests on independent streams cannot at these sizes."""
    setup = pp.workloads.c1_setup(photons=15_000_000, seed=11)
    rf, cf, nf, _ = gpu_run(pp, setup, precise_math=0)
    assert rf == 0
    want, _ = orc.Run.from_setup(setup).propagate(precision="f64")
    kf, kw = set(cf["photon_index"].tolist()), set(want["photon_index"].tolist())
    n_fast_only, n_f64_only = len(kf - kw), len(kw - kf)
    n = n_fast_only + n_f64_only
    assert n < 0.05 * len(kw)
    assert abs(n_fast_only - n_f64_only) <= 3.0 * np.sqrt(max(n, 1)) + 2, (n_fast_only,
                                                                            n_f64_only)


def _cascades_inside_detector(pp, seed, n_sources=6, photons=1_000_000, rng_seed=19):
    """Extended Cherenkov cascades (a = 2.0, b = 0.63, lrad = 0.36 m) 3-10 m
    from modules of the C1 detector, pointing in random directions."""
    targets, _ = pp.workloads.detector_400()
    rng = np.random.default_rng(rng_seed)
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    srcs = []
    for _ in range(n_sources):
        t = np.asarray(targets[rng.integers(len(targets))].shape.position)
        v = rng.normal(size=3)
        v *= rng.uniform(3.0, 10.0) / np.linalg.norm(v)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        srcs.append(pp.ExtendedCherenkovEmitter(list(t + v), list(d), 0.0, photons, lp))
    medium = pp.CascadiaMediumProperties(0.95, 0.2, 1.0, 1.0)
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), medium)
    return pp.PhotonPropSetup(srcs, targets, medium, spec, seed)


@pytest.mark.gpu
def test_cascade_emitters_statistics(pp, orc, gpu_ctx):
    """Cascades among the C1 modules: on the same random streams the fast
    kernel and the FP64 oracle disagree on as many photons one way as the
    other (sign test), and on independent streams the per-module counts and
    the arrival times agree with the FP32 oracle (chi-square, KS; p > 0.01)."""
    setup = _cascades_inside_detector(pp, seed=71)
    rc, cols, nh, nsim = gpu_run(pp, setup)
    assert rc == 0 and nsim == 6 * 1_000_000
    run = orc.Run.from_setup(setup)
    keys_f = set(zip(cols["source_index"].tolist(), cols["photon_index"].tolist()))
    keys_w = set()
    for src in range(len(setup.sources)):
        w, _ = run.propagate(src, precision="f64")
        keys_w |= set(zip(w["source_index"].tolist(), w["photon_index"].tolist()))
    n_f, n_w = len(keys_f - keys_w), len(keys_w - keys_f)
    assert n_f + n_w < 0.05 * len(keys_w)
    assert abs(n_f - n_w) <= 3.0 * np.sqrt(max(n_f + n_w, 1)) + 2, (n_f, n_w)
    other = _cascades_inside_detector(pp, seed=72)
    want, _, _ = orc.Run.from_setup(other).propagate_all()
    n_mod = len(setup.targets)
    g = np.bincount(cols["module_index"] - 1, minlength=n_mod)
    o = np.bincount(want["module_index"] - 1, minlength=n_mod)
    chi2, dof, p = two_sample_poisson_chi2(g, o)
    assert g.sum() > 1500 and p > P_MIN, (g.sum(), chi2, dof, p)
    assert stats.ks_2samp(cols["time"], want["time"]).pvalue > P_MIN


@pytest.mark.gpu
def test_c0_arrival_time_histogram(pp, orc, gpu_ctx):
    """The README example (one module at 10 m, 450 nm): the hit count and the
    arrival-time histogram in 1 ns bins on 0-500 ns agree with the oracle
    (two-sample chi-square p > 0.01; 1e7 photons, 100x the example's 1e5, so
    that the histogram has power)."""
    photons = 10_000_000
    setup_g = pp.workloads.c0_setup(photons, seed=60)
    setup_o = pp.workloads.c0_setup(photons, seed=61)
    rc, cols, nh, nsim = gpu_run(pp, setup_g)
    assert rc == 0 and nsim == photons
    want, _ = orc.Run.from_setup(setup_o).propagate()
    assert abs(nh - len(want)) / np.sqrt(nh + len(want)) < 4
    edges = np.arange(0.0, 501.0, 1.0)
    hg, _ = np.histogram(cols["time"], edges)
    ho, _ = np.histogram(want["time"], edges)
    assert hg.sum() > 1000
    chi2, dof, p = two_sample_poisson_chi2(hg, ho)
    assert p > P_MIN, (chi2, dof, p)
