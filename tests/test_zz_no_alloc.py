"""pp_propagate_static -- the entry point for callers that cannot call
cudaMalloc (another framework's pool owns the device memory, or memory use is
fixed at start-up).  It must give the same hits as the context-based
pp_propagate, twice in a row, while taking all of its scratch from the
library's static device array, and leave the device's free memory unchanged.

Collected last on purpose: if it fails, a run that stops at the first
failure has already run every other test."""
import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu

FIELDS = ("position", "direction", "initial_direction", "wavelength", "time", "dist_travelled",
          "abs_weight", "module_index", "n_steps", "source_index", "photon_index")


def _medium_struct(pp, tables):
    arrs = [np.ascontiguousarray(a, np.float32) for a in
            (tables.scattering_length, tables.group_velocity, tables.absorption_length,
             tables.phase_refractive_index)]
    m = pp._lib.pp_medium()
    m.wl_min, m.wl_step, m.n_knots = tables.wl_min, tables.wl_step, arrs[0].shape[0]
    fp = ctypes.POINTER(ctypes.c_float)
    m.scattering_length, m.group_velocity, m.absorption_length, m.phase_refractive_index = (
        a.ctypes.data_as(fp) for a in arrs)
    m.hg_g, m.es_b, m.hg_weight = tables.hg_g, tables.es_b, tables.hg_weight
    return m, arrs


def _static_call(pp, setup, d_hits, capacity, n_steps=15):
    """One call of the new entry point through the C ABI; returns (rc, counters)."""
    lib = pp._lib.load()
    m, keep = _medium_struct(pp, setup.medium_tables())
    fp = ctypes.POINTER(ctypes.c_float)
    if setup.spectrum_knots is not None:
        knots = np.ascontiguousarray(setup.spectrum_knots, np.float32)
        kp, nk, mono = knots.ctypes.data_as(fp), knots.shape[0], 0.0
    else:
        knots, kp, nk, mono = None, None, 0, setup.mono_wavelength
    track = (np.ascontiguousarray(setup.track_quantiles(), np.float32)
             if setup.needs_track_smear() else None)
    tp = track.ctypes.data_as(fp) if track is not None else None
    spheres = setup.sphere_records()
    srcs = setup.source_records()
    ctr = pp._lib.pp_counters()
    rc = lib.pp_propagate_static(ctypes.byref(m), kp, nk, mono, tp,
                                 0 if track is None else track.shape[0], spheres,
                                 len(setup.targets), 0.0, srcs, len(setup.sources), setup.seed,
                                 n_steps, setup.photon_scaling, ctypes.c_void_p(d_hits), capacity,
                                 ctypes.byref(ctr), None)
    return rc, ctr


def _sorted(cols):
    order = np.lexsort((cols["photon_index"], cols["source_index"]))
    return {k: np.asarray(cols[k])[order] for k in FIELDS}


def _records_to_columns(pp, raw, n):
    rec = raw.view(np.dtype(pp._lib.HIT_RECORD_DTYPE))[:n]
    return {k: rec[k] for k in FIELDS}


@pytest.mark.parametrize("which", ["detector_400", "cherenkov_sources"])
def test_static_scratch_matches_context_entry_point(pp, gpu_ctx, which):
    torch = pytest.importorskip("torch")
    if which == "detector_400":
        setup = pp.workloads.c1_setup(photons=400_000, seed=5)
    else:
        setup = pp.workloads.c2_setup(n_sources=16, scale=0.3)
    capacity = 200_000

    # existing entry point (context-owned buffers)
    ctx = pp.get_context(0)
    setup.upload(ctx)
    rc, n_ref, sim_ref = ctx.propagate(setup.source_records(), len(setup.sources), setup.seed, 15,
                                       setup.photon_scaling, capacity)
    assert rc == 0 and n_ref > 10
    want = _sorted(ctx.fetch_hits(n_ref))

    raw = torch.empty(capacity * 80, dtype=torch.uint8, device="cuda")
    for call in range(2):  # two calls in a row share the static array
        raw.fill_(0xff)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        rc, ctr = _static_call(pp, setup, raw.data_ptr(), capacity)
        free_after = torch.cuda.mem_get_info()[0]
        assert rc == 0, pp._lib.last_error()
        if call == 1:  # the first call may load the module's image; later ones allocate nothing
            assert free_after == free_before, (free_before, free_after)
        assert ctr.n_hits == n_ref and ctr.n_ph_sim == sim_ref and ctr.err_flags == 0
        got = _sorted(_records_to_columns(pp, raw.cpu().numpy(), int(ctr.n_hits)))
        for k in FIELDS:
            np.testing.assert_array_equal(got[k], want[k], err_msg=f"{k}, call {call}")


def test_static_scratch_limits_and_overflow(pp, gpu_ctx):
    torch = pytest.importorskip("torch")
    setup = pp.workloads.c0_setup(400_000)
    raw = torch.empty(100_000 * 80, dtype=torch.uint8, device="cuda")
    rc, ctr = _static_call(pp, setup, raw.data_ptr(), 100_000)
    assert rc == 0 and ctr.n_hits > 10
    rc, ctr2 = _static_call(pp, setup, raw.data_ptr(), int(ctr.n_hits) - 1)
    assert rc == pp._lib.PP_ERR_OVERFLOW and ctr2.n_hits == ctr.n_hits
    # a medium table too large for the 8 MiB array is refused with a clear error
    lib = pp._lib.load()
    n = 600_000
    big = np.ones(n, np.float32)
    fp = ctypes.POINTER(ctypes.c_float)
    m = pp._lib.pp_medium()
    m.wl_min, m.wl_step, m.n_knots = 300.0, 0.001, n
    m.scattering_length = m.group_velocity = m.absorption_length = big.ctypes.data_as(fp)
    m.phase_refractive_index = big.ctypes.data_as(fp)
    m.hg_g, m.es_b, m.hg_weight = 0.9, 0.835, 0.8
    ctr3 = pp._lib.pp_counters()
    rc = lib.pp_propagate_static(ctypes.byref(m), None, 0, 450.0, None, 0,
                                 setup.sphere_records(), 1, 0.0, setup.source_records(), 1, 1, 15,
                                 1.0, ctypes.c_void_p(raw.data_ptr()), 100_000, ctypes.byref(ctr3),
                                 None)
    assert rc == pp._lib.PP_ERR_INVALID
    assert "MiB static array" in pp._lib.last_error()
