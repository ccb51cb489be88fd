"""CUDA path vs the CPU oracle, photon by photon (replay) and statistically.
All GPU calls go through the C ABI (ctypes)."""
import os
import sys

import numpy as np
import pytest
from scipy import stats

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from replay import compare, oracle_columns, spheres_of  # noqa: E402

pytestmark = pytest.mark.gpu


def gpu_run(pp, setup, n_steps=15, capacity=None, **tuning):
    ctx = pp.get_context(0)
    old = ctx.get_tuning()
    try:
        if tuning:
            ctx.set_tuning(**tuning)
        setup.upload(ctx)
        recs = setup.source_records()
        cap = capacity if capacity is not None else sum(
            pp.source_photons(s.photons, setup.photon_scaling) for s in setup.sources)
        rc, nh, nsim = ctx.propagate(recs, len(setup.sources), setup.seed, n_steps,
                                     setup.photon_scaling, cap)
        cols = ctx.fetch_hits(nh) if rc == 0 else None
        return rc, cols, nh, nsim
    finally:
        ctx.set_tuning(block_threads=old.block_threads,
                       photons_per_thread=old.photons_per_thread,
                       ctas_per_sm=old.ctas_per_sm, precise_math=old.precise_math,
                       cell_size=old.cell_size, grid_in_global=old.grid_in_global,
                       target_loop=old.target_loop)


def test_philox_device_matches_oracle(pp, orc, gpu_ctx):
    rng = np.random.default_rng(5)
    ctr = rng.integers(0, 2 ** 32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    for key in ((0, 0), (1, 0), (0xdeadbeef, 0x12345678)):
        dev = pp.debug_philox(ctr, *key)
        for i in range(0, 4096, 97):
            assert tuple(dev[i]) == tuple(orc.philox(ctr[i], key))


@pytest.mark.parametrize("precise", [1, 0])
def test_c0_replay(pp, orc, gpu_ctx, precise):
    setup = pp.workloads.c0_setup(400_000)
    rc, cols, nh, nsim = gpu_run(pp, setup, precise_math=precise)
    assert rc == 0 and nsim == 400_000
    want, st = orc.Run.from_setup(setup).propagate()
    assert st.n_ph_sim == nsim
    s = compare(cols, oracle_columns(want), spheres_of(setup),
                mode="precise" if precise else "fast")
    assert s["matched"] > 50


@pytest.mark.parametrize("precise", [1, 0])
def test_c1_detector_replay(pp, orc, gpu_ctx, precise):
    setup = pp.workloads.c1_setup(photons=300_000, seed=2)
    rc, cols, nh, nsim = gpu_run(pp, setup, precise_math=precise)
    assert rc == 0 and nsim == 300_000
    want, st = orc.Run.from_setup(setup).propagate()
    s = compare(cols, oracle_columns(want), spheres_of(setup),
                mode="precise" if precise else "fast")
    assert s["matched"] > 20, s


def test_launch_shape_and_grid_invariance(pp, gpu_ctx):
    """Per-photon random streams: the hit set does not depend on the block
    size, photons per thread, grid cell size or where the grid is read from --
    nor on the culling at all: target_loop = 1 tests every sphere at every
    step in index order (the reference's own loop, src/photon_prop_cuda.jl:
    497-506) and must find exactly the same hits as the culled walk."""
    setup = pp.workloads.c1_setup(photons=400_000, seed=3)
    base = None
    for tun in (dict(block_threads=256, photons_per_thread=8),
                dict(block_threads=1024, photons_per_thread=2),
                dict(block_threads=256, photons_per_thread=8, target_loop=1),
                dict(block_threads=128, photons_per_thread=1),
                dict(block_threads=512, photons_per_thread=16, grid_in_global=1),
                dict(block_threads=256, photons_per_thread=4, cell_size=12.0),
                dict(block_threads=256, photons_per_thread=4, cell_size=60.0)):
        rc, cols, nh, nsim = gpu_run(pp, setup, **tun)
        assert rc == 0
        order = np.argsort(cols["photon_index"])
        cur = {k: v[order] for k, v in cols.items()}
        if base is None:
            base = cur
            assert nh > 10
            continue
        for k in base:
            np.testing.assert_array_equal(cur[k], base[k], err_msg=f"{k} with {tun}")


EMITTERS = {
    "extended_cherenkov": lambda pp: pp.ExtendedCherenkovEmitter(
        [3.0, -2.0, 1.0], [0.6, 0.0, 0.8], 0.0, 200_000, pp.LongitudinalParameterisation(2.0, 0.63, 0.36)),
    "extended_cherenkov_nosmear": lambda pp: pp.ExtendedCherenkovEmitterNoSmear(
        [3.0, -2.0, 1.0], [0.0, 0.6, 0.8], 5.0, 200_000, pp.LongitudinalParameterisation(0.7, 0.63, 0.36)),
    "custom_smear": lambda pp: pp.ExtendedCherenkovEmitterCustomSmear(
        [3.0, -2.0, 1.0], [0.6, 0.0, 0.8], 0.0, 200_000, pp.LongitudinalParameterisation(2.0, 0.63, 0.36),
        3.0, 0.4),
    "pointlike_cherenkov": lambda pp: pp.PointlikeCherenkovEmitter(
        [0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 200_000),
    "cherenkov_track": lambda pp: pp.CherenkovTrackEmitter(
        [-20.0, 0.0, 5.0], [1.0, 0.0, 0.0], 0.0, 40.0, 200_000),
    "time_range": lambda pp: pp.PointlikeTimeRangeEmitter([0.0, 0.0, 0.0], (10.0, 30.0), 200_000),
    "collimated": lambda pp: pp.CollimatedIsotropicEmitter([0.0, 0.0, 0.0], 0.0, 200_000, 0.9),
    "pencil": lambda pp: pp.PencilEmitter([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.05, 0.0, 200_000),
    "axicone": lambda pp: pp.AxiconeEmitter([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 200_000, 0.2, 0.02),
}


@pytest.mark.parametrize("name", sorted(EMITTERS))
def test_emitter_replay(pp, orc, gpu_ctx, name):
    med = pp.CascadiaMediumProperties()
    targets = [pp.HomogeneousDetector(pp.Spherical(p, 1.0), 1.0, i + 1)
               for i, p in enumerate([[0, 0, 10], [8, 0, 6], [-6, 5, 8], [0, -9, 4], [5, 5, -5]])]
    spec = pp.make_cherenkov_spectrum((300.0, 800.0), med)
    setup = pp.PhotonPropSetup([EMITTERS[name](pp)], targets, med, spec, 9)
    rc, cols, nh, nsim = gpu_run(pp, setup, precise_math=1)
    assert rc == 0
    want, st = orc.Run.from_setup(setup).propagate()
    assert nsim == st.n_ph_sim
    s = compare(cols, oracle_columns(want), spheres_of(setup))
    assert s["matched"] > 100, s


def test_custom_smear_tables_replay(pp, orc, gpu_ctx):
    """Sources drawing their track smear from different tables in one launch."""
    med = pp.CascadiaMediumProperties()
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    srcs = [pp.ExtendedCherenkovEmitter([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 150_000, lp),
            pp.ExtendedCherenkovEmitterCustomSmear([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 150_000,
                                                   lp, 1e3, 1e-3),
            pp.ExtendedCherenkovEmitterCustomSmear([0.0, 0.0, 0.0], [0.0, 0.0, 1.0], 0.0, 150_000,
                                                   lp, 0.5, 0.5)]
    targets = [pp.HomogeneousDetector(pp.Spherical(p, 1.0), 1.0, i + 1)
               for i, p in enumerate([[0, 0, 10], [8, 0, 6], [-6, 5, 8], [0, -9, 4], [5, 5, -5]])]
    setup = pp.PhotonPropSetup(srcs, targets, med, pp.make_cherenkov_spectrum((300.0, 800.0), med),
                               5)
    assert setup.track_table_stack().shape[0] == 3
    rc, cols, nh, nsim = gpu_run(pp, setup, precise_math=1)
    assert rc == 0
    want, sim, _ = orc.Run.from_setup(setup).propagate_all()
    assert nsim == sim == 450_000
    s = compare(cols, oracle_columns(want), spheres_of(setup))
    assert s["matched"] > 300, s
    for k in range(3):
        assert (cols["source_index"] == k).sum() > 50, k


def test_many_sources_one_launch(pp, orc, gpu_ctx):
    """A work queue over sources with uneven photon counts."""
    setup = pp.workloads.c2_setup(n_sources=24, scale=0.02)
    rc, cols, nh, nsim = gpu_run(pp, setup, precise_math=1)
    assert rc == 0
    want, sim, steps = orc.Run.from_setup(setup).propagate_all()
    assert nsim == sim
    compare(cols, oracle_columns(want), spheres_of(setup))


def test_overflow_raises(pp, gpu_ctx):
    setup = pp.workloads.c0_setup(400_000)
    rc, cols, nh, nsim = gpu_run(pp, setup)
    assert rc == 0 and nh > 10
    rc2, _, nh2, _ = gpu_run(pp, setup, capacity=nh - 1)
    assert rc2 == pp._lib.PP_ERR_OVERFLOW
    rc3, cols3, nh3, _ = gpu_run(pp, setup, capacity=nh)
    assert rc3 == 0 and nh3 == nh
    with pytest.raises(pp.PhotonPropOOMException):
        pp.propagate_photons(setup, pp.HitBuffers(nh - 1))


def test_staging_wait_times_out_and_context_recovers(pp, gpu_ctx):
    """The kernel's one wait (the TMA staging of the culling tables, bounded by
    %globaltimer) is made to run out: the diagnostic arms the barrier and
    issues no copy, with a 1 ms bound.  Every CTA must raise PP_FLAG_TIMEOUT
    and return, the call must report PP_ERR_TIMEOUT, and the next normal
    launch on the same context must give the same hits as before."""
    setup = pp.workloads.c1_setup(photons=200_000, seed=6)
    rc, cols, nh, nsim = gpu_run(pp, setup)
    assert rc == 0 and nh > 0
    ctx = pp.get_context(0)
    lib = pp._lib.load()
    rc = lib.pp_debug_staging_timeout(ctx.ptr, 1_000_000)
    assert rc == pp._lib.PP_ERR_TIMEOUT, (rc, pp._lib.last_error())
    assert "timed out" in pp._lib.last_error()
    assert lib.pp_debug_staging_timeout(ctx.ptr, 10) == pp._lib.PP_ERR_INVALID
    rc2, cols2, nh2, nsim2 = gpu_run(pp, setup)
    assert rc2 == 0 and nh2 == nh and nsim2 == nsim
    o1, o2 = np.argsort(cols["photon_index"]), np.argsort(cols2["photon_index"])
    np.testing.assert_array_equal(cols["position"][o1], cols2["position"][o2])


def test_propagate_photons_table(pp, gpu_ctx):
    setup = pp.workloads.c0_setup(300_000)
    t = pp.propagate_photons(setup)
    assert t.n_ph_sim == 300_000
    n = t.nrow
    assert n > 20
    assert set(t["module_id"]) == {1}
    np.testing.assert_allclose(t["base_weight"], 300_000 / 300_000)
    # in-kernel absorption weight equals the host FP64 formula
    abs_len = setup.medium.absorption_length(t["wavelength"].astype(np.float64))
    np.testing.assert_allclose(t["abs_weight"], np.exp(-t["dist_travelled"] / abs_len), rtol=2e-6)
    assert np.all(t["time"] > 0) and t["time"].dtype == np.float64
    # a second call with the same seed is identical (up to row order)
    t2 = pp.propagate_photons(setup)
    o1, o2 = np.argsort(t["photon_index"]), np.argsort(t2["photon_index"])
    np.testing.assert_array_equal(t["position"][o1], t2["position"][o2])


def test_c0_statistics_vs_oracle(pp, orc, gpu_ctx):
    """Fast-math kernel, independent seeds: hit counts within Poisson, arrival
    time and wavelength distributions pass KS against the oracle."""
    setup_g = pp.workloads.c0_setup(2_000_000, seed=11)
    setup_o = pp.workloads.c0_setup(2_000_000, seed=12)
    rc, cols, nh, nsim = gpu_run(pp, setup_g)
    want, st = orc.Run.from_setup(setup_o).propagate()
    n_o = len(want)
    z = (nh - n_o) / np.sqrt(nh + n_o)
    assert abs(z) < 4, (nh, n_o)
    assert stats.ks_2samp(cols["time"], want["time"]).pvalue > 0.01
    setup_g = pp.workloads.c1_setup(photons=3_000_000, seed=21)
    setup_o = pp.workloads.c1_setup(photons=3_000_000, seed=21)
    setup_o.seed = 22
    rc, cols, nh, nsim = gpu_run(pp, setup_g)
    want, _ = orc.Run.from_setup(setup_o).propagate()
    assert stats.ks_2samp(cols["wavelength"], want["wavelength"]).pvalue > 0.01
    assert abs(nh - len(want)) / np.sqrt(nh + len(want)) < 4


def test_graph_launch_matches_plain_launch(pp, gpu_ctx):
    torch = pytest.importorskip("torch")
    setup = pp.workloads.c1_setup(photons=500_000, seed=4)
    ctx = pp.get_context(0)
    setup.upload(ctx)
    recs = setup.source_records()
    ctx.set_sources(recs, len(setup.sources), 1.0)
    cap = 500_000
    hits = torch.zeros(cap * 80 // 4, dtype=torch.int32, device="cuda")
    ctr = torch.zeros(12, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    res = []
    for graph in (False, True, True):
        with torch.cuda.stream(s):
            ctx.launch(setup.seed, 15, hits.data_ptr(), cap, ctr.data_ptr(), s.cuda_stream,
                       graph=graph)
        s.synchronize()
        c = ctr.cpu().numpy().view(np.uint64)
        n = int(c[0])
        rec = hits.cpu().numpy().view(np.dtype(pp._lib.HIT_RECORD_DTYPE))[:n]
        res.append((int(c[1]), int(c[2]), np.sort(rec["photon_index"]), n))
    assert res[0][0] == 500_000
    for r in res[1:]:
        assert r[0] == res[0][0] and r[1] == res[0][1] and r[3] == res[0][3]
        np.testing.assert_array_equal(r[2], res[0][2])


def test_photon_steps_counter(pp, orc, gpu_ctx):
    torch = pytest.importorskip("torch")
    setup = pp.workloads.c0_setup(100_000)
    ctx = pp.get_context(0)
    setup.upload(ctx)
    ctx.set_sources(setup.source_records(), 1, 1.0)
    hits = torch.zeros(100_000 * 20, dtype=torch.int32, device="cuda")
    ctr = torch.zeros(12, dtype=torch.int32, device="cuda")
    ctx.launch(1, 15, hits.data_ptr(), 100_000, ctr.data_ptr(), 0)
    torch.cuda.synchronize()
    c = ctr.cpu().numpy().view(np.uint64)
    _, st = orc.Run.from_setup(setup).propagate()
    assert int(c[1]) == st.n_ph_sim
    assert abs(int(c[2]) - st.photon_steps) <= 15 * 5  # grazing hits may differ


def test_validation_formula(pp, gpu_ctx):
    """The reference's loose check (examples/validation.jl:300-306): photons
    from an isotropic source reaching a sphere of radius r at distance d follow
    norm * N r^2 / (4 d^2) * exp(-d / L) -- fitted here over five distances
    (absorption-weighted counts, as the reference's sphere hits)."""
    med = pp.CascadiaMediumProperties()
    dists = np.array([8.0, 15.0, 25.0, 40.0, 60.0])
    dirs = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0], [-1, 0, 0], [0, -1, 0]], float)
    targets = [pp.HomogeneousDetector(pp.Spherical(list(d * u), 1.0), 1.0, i + 1)
               for i, (d, u) in enumerate(zip(dists, dirs))]
    n = 50_000_000
    src = pp.PointlikeIsotropicEmitter([0.0, 0.0, 0.0], 0.0, n)
    setup = pp.PhotonPropSetup([src], targets, med,
                               pp.make_cherenkov_spectrum((300.0, 800.0), med), 2)
    table = pp.propagate_photons(setup)
    w = np.array([table["total_weight"][table["module_id"] == i + 1].sum() for i in range(5)])
    geo = n * 1.0 / (4 * dists ** 2)
    slope, icpt = np.polyfit(dists, np.log(w / geo), 1)
    L, norm = -1.0 / slope, np.exp(icpt)
    model = norm * geo * np.exp(-dists / L)
    assert 10.0 < L < 60.0, L
    assert 0.3 < norm < 3.0, norm
    assert np.max(np.abs(w / model - 1)) < 0.3, w / model


def test_c1_full_size_properties(pp, orc, gpu_ctx):
    """At the benchmark's size (C1, 1e8 photons): the hit set is bitwise the
    same for two launch shapes, the union of four photon-range shards is
    bitwise the single run, and the hit rate agrees with the oracle's on the
    run's first 1.5e6 photons."""
    import copy
    setup = pp.workloads.c1_setup(photons=100_000_000, seed=1)
    n = pp.source_photons(setup.sources[0].photons, setup.photon_scaling)
    cap = 1_000_000

    def sorted_cols(cols):
        o = np.argsort(cols["photon_index"])
        return {k: v[o] for k, v in cols.items()}
    rc, base, nh, nsim = gpu_run(pp, setup, capacity=cap)
    assert rc == 0 and nsim == n and nh > 5000
    base = sorted_cols(base)
    rc, other, _, _ = gpu_run(pp, setup, capacity=cap, block_threads=256, photons_per_thread=8,
                              cell_size=25.0)
    other = sorted_cols(other)
    for k in base:
        np.testing.assert_array_equal(other[k], base[k], err_msg=k)
    parts = []
    src = setup.sources[0]
    for r in range(4):
        lo, hi = n * r // 4, n * (r + 1) // 4
        c = copy.copy(src)
        c.photons, c.first_photon = hi - lo, lo
        s = copy.copy(setup)
        s.sources = [c]
        rc, cols, _, sim = gpu_run(pp, s, capacity=cap)
        assert rc == 0 and sim == hi - lo
        parts.append(cols)
    merged = sorted_cols({k: np.concatenate([p[k] for p in parts]) for k in base})
    for k in base:
        np.testing.assert_array_equal(merged[k], base[k], err_msg=k)
    # the oracle on the first 1.5e6 photons of the same run
    m = 1_500_000
    c = copy.copy(src)
    c.photons = m
    s = copy.copy(setup)
    s.sources = [c]
    want, sim, _ = orc.Run.from_setup(s).propagate_all()
    assert sim == m
    first = {k: v[base["photon_index"] < m] for k, v in base.items()}
    st = compare(first, oracle_columns(want), spheres_of(setup), mode="fast")
    assert st["matched"] > 100, st
    rate_all, rate_or = nh / n, len(want) / m
    assert abs(rate_all - rate_or) < 5 * np.sqrt(rate_or / m), (rate_all, rate_or)


def test_public_autotune_keeps_results(pp, gpu_ctx):
    """pp.autotune tunes the context that propagate_photons uses; the hit
    table is the same before and after (per-photon random streams)."""
    setup = pp.workloads.c1_setup(photons=2_000_000, seed=2)
    before = pp.propagate_photons(setup)
    orig = gpu_ctx.get_tuning()
    try:
        t = pp.autotune(setup, 15, sample_photons=1_000_000)
        assert 64 <= t["block_threads"] <= 1024 and t["block_threads"] % 32 == 0
        assert t["photons_per_thread"] >= 1 and t["cell_size"] > 0 and t["photons_per_s"] > 0
        after = pp.propagate_photons(setup)
    finally:
        gpu_ctx.set_tuning(block_threads=orig.block_threads,
                           photons_per_thread=orig.photons_per_thread,
                           cell_size=orig.cell_size, safety_cell=orig.safety_cell,
                           ctas_per_sm=orig.ctas_per_sm)
    assert after.nrow == before.nrow > 0
    o1, o2 = np.argsort(before["photon_index"]), np.argsort(after["photon_index"])
    for k in ("position", "direction", "time", "module_id", "n_steps"):
        np.testing.assert_array_equal(before[k][o1], after[k][o2], err_msg=k)
