"""C ABI and host logic without a GPU: the library loads, exports every
symbol the header declares, rejects bad input, and the host-side mirror of
the reference API computes what the reference computes."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu

HEADER = os.path.join(ROOT, "include", "pp_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"PP_API\s+[\w\s\*]+?\b(pp_\w+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("pp_create", "pp_destroy", "pp_set_medium", "pp_set_spectrum", "pp_set_targets",
              "pp_propagate", "pp_launch", "pp_launch_graph", "pp_last_error", "pp_autotune"):
        assert s in syms


def test_library_exports_every_declared_symbol(pp):
    lib = ctypes.CDLL(pp._lib.lib_path())
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    # and the Python binding knows all of them
    assert set(declared_symbols()) <= set(pp._lib.SIGNATURES), \
        set(declared_symbols()) - set(pp._lib.SIGNATURES)


def test_struct_layouts_match_header(pp):
    L = pp._lib
    assert ctypes.sizeof(L.pp_source) == 96
    assert ctypes.sizeof(L.pp_sphere) == 16
    assert ctypes.sizeof(L.pp_hit_record) == 80
    assert ctypes.sizeof(L.pp_counters) == 48
    assert L.pp_hit_record.time.offset == 64
    assert L.pp_hit_record.module_index.offset == 28  # in the first 32-byte sector
    assert L.pp_source.first_photon.offset == 80
    assert np.dtype(L.HIT_RECORD_DTYPE).itemsize == 80


def test_ctypes_layouts_match_the_c_compiler(pp, orc):
    """Every ABI struct's size and the offsets the library relies on, as the C
    compiler lays them out from the header, equal the ctypes mirror's."""
    L = pp._lib
    C = orc.load()
    for name in ("pp_source", "pp_sphere", "pp_medium", "pp_tuning", "pp_hit_record",
                 "pp_counters", "pp_target", "pp_pmt_target", "pp_pom_model", "pp_dom_model",
                 "pp_multipmt_model", "pp_detection_models", "pp_hits"):
        assert C.ppo_abi_layout(name.encode()) == ctypes.sizeof(getattr(L, name)), name
    for name, field in (("pp_source", "smear_table"), ("pp_source", "first_photon"),
                        ("pp_medium", "phase_kind"), ("pp_medium", "hg_g"),
                        ("pp_hit_record", "time"), ("pp_hit_record", "module_index"),
                        ("pp_dom_model", "polymax"), ("pp_dom_model", "apply_wl_acceptance"),
                        ("pp_dom_model", "wl"), ("pp_multipmt_model", "pmt_dir"),
                        ("pp_multipmt_model", "qe"), ("pp_pom_model", "pmt_dir"),
                        ("pp_pom_model", "pmt_group"), ("pp_detection_models", "multipmt")):
        got = C.ppo_abi_layout(f"{name}.{field}".encode())
        assert got == getattr(getattr(L, name), field).offset, (name, field)
    assert C.ppo_abi_layout(b"pp_nothing") == -1


def test_detection_argument_checks(pp):
    """pp_make_hits_from_photons_models rejects bad modules and models before
    touching a device (and n = 0 is a no-op)."""
    L = pp._lib
    lib = L.load()
    fake = ctypes.c_void_p(256)  # never dereferenced: validation comes first
    tg = (L.pp_pmt_target * 1)()
    tg[0].radius = 0.3

    def call(models, n=1):
        return lib.pp_make_hits_from_photons_models(fake, n, tg, 1, ctypes.byref(models), 0,
                                                    fake, None, None)
    none = L.pp_detection_models()
    for kind, msg in ((L.PP_PMT_POM, "without its model"), (L.PP_PMT_DOM, "without its model"),
                      (L.PP_PMT_MULTIPMT, "without its model"), (9, "unknown module kind")):
        tg[0].kind = kind
        assert call(none) == L.PP_ERR_INVALID and msg in L.last_error(), kind
    tg[0].kind = L.PP_PMT_DOM
    dom = pp.dom.dom_model()
    dom.n_poly = 0
    models = L.pp_detection_models(dom=ctypes.pointer(dom))
    assert call(models) == L.PP_ERR_INVALID and "bad DOM tables" in L.last_error()
    tg[0].kind = L.PP_PMT_MULTIPMT
    mp = pp.generic_multipmt.multipmt_model([pp.make_generic_multipmt_om([0, 0, 0], 0.2, 1)])
    mp.n_pmt = L.PP_MULTIPMT_MAX_PMTS + 1
    models = L.pp_detection_models(multipmt=ctypes.pointer(mp))
    assert call(models) == L.PP_ERR_INVALID and "bad multi-PMT tables" in L.last_error()
    mp.n_pmt = 20
    tg[0].radius = 0.0
    assert call(models) == L.PP_ERR_INVALID and "radius" in L.last_error()
    tg[0].radius = 0.2
    assert call(models, n=0) == L.PP_OK


def test_version_and_error_text(pp):
    lib = pp._lib.load()
    assert lib.pp_version() == 1
    assert lib.pp_last_error(None, 0) >= 0


@pytest.mark.skipif(has_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly(pp):
    lib = pp._lib.load()
    p = ctypes.c_void_p()
    assert lib.pp_create(ctypes.byref(p), 0) == pp._lib.PP_ERR_NO_DEVICE
    assert "no CUDA device" in pp._lib.last_error()
    with pytest.raises(pp._lib.PPError):
        pp.Context(0)
    with pytest.raises(pp._lib.PPError):
        pp.propagate_photons(pp.workloads.c0_setup(10))


def test_null_arguments_rejected(pp):
    lib = pp._lib.load()
    assert lib.pp_create(None, 0) == pp._lib.PP_ERR_INVALID
    assert lib.pp_set_medium(None, None) == pp._lib.PP_ERR_INVALID
    assert lib.pp_propagate(None, None, 0, 1, 15, 1.0, None, 0, None, None) == \
        pp._lib.PP_ERR_INVALID
    assert lib.pp_destroy(None) == 0


def test_setup_spectrum_forms(pp):
    med = pp.CascadiaMediumProperties()
    src = pp.PointlikeIsotropicEmitter([0, 0, 0], 0.0, 100)
    tgt = pp.HomogeneousDetector(pp.Spherical([0, 0, 10], 0.3), 1.0, 7)
    a = pp.PhotonPropSetup([src], [tgt], med, pp.make_monochromatic_spectrum(450.0), 1)
    b = pp.PhotonPropSetup([src], [tgt], med, pp.Monochromatic(450.0), 1)  # README form
    assert a.mono_wavelength == b.mono_wavelength == 450.0
    c = pp.PhotonPropSetup([src], [tgt], med, pp.make_cherenkov_spectrum((300.0, 800.0), med), 1,
                           spectrum_interp_steps=300)
    assert c.spectrum_knots.shape == (300,) and c.mono_wavelength is None
    lo, hi = c.wavelength_range()
    t = c.medium_tables()
    assert t.wl_min <= lo and t.wl_min + t.wl_step * (t.n_knots - 1) >= hi
    assert not c.needs_track_smear()
    recs = c.source_records()
    assert recs[0].kind == 0 and recs[0].photons == 100 and recs[0].first_photon == 0


def test_track_smear_table(pp):
    q = pp.propsetup.PhotonPropSetup(
        [pp.ExtendedCherenkovEmitter([0, 0, 0], [0, 0, 1], 0.0, 10,
                                     pp.LongitudinalParameterisation(2.0, 0.63, 0.36))],
        [], pp.CascadiaMediumProperties(), pp.make_monochromatic_spectrum(400.0), 1
    ).track_quantiles()
    assert q.shape == (4096,) and q[0] == -1.0 and q[-1] == 1.0
    assert np.all(np.diff(q) >= 0)
    from scipy import stats
    # cos = 2 Beta(1.776, 0.164) - 1
    mean = 2 * 1.776 / (1.776 + 0.164) - 1
    u = (np.arange(200000) + 0.5) / 200000
    assert np.interp(u, np.linspace(0, 1, 4096), q).mean() == pytest.approx(mean, abs=2e-3)


def test_longitudinal_parameterisation_from_energy(pp):
    med = pp.CascadiaMediumProperties()
    lp = pp.LongitudinalParameterisation.from_energy(1.0, med, "EMinus")
    assert lp.a == pytest.approx(2.01849) and lp.b == pytest.approx(0.63207)
    assert lp.lrad == pytest.approx(0.356, abs=0.005)
    lp2 = pp.LongitudinalParameterisation.from_energy(1e3, med, "EMinus")
    assert lp2.a == pytest.approx(2.01849 + 3 * 1.45469)


def test_module_id_remap_and_weights(pp):
    """module_id = ids[module_index]; base_weight = sum(photons)/n_ph_sim;
    total = base * abs (src/processing.jl:67-74)."""
    tg = [pp.HomogeneousDetector(pp.Spherical([0, 0, z], 0.3), 1.0, mid)
          for z, mid in ((10, 17), (20, 3), (30, 99))]
    ids = pp.targets.module_ids(tg)
    assert ids.dtype == np.uint16
    assert list(ids[np.array([1, 3, 2, 1]) - 1]) == [17, 99, 3, 17]
    med = pp.CascadiaMediumProperties()
    setup = pp.PhotonPropSetup([pp.PointlikeIsotropicEmitter([0, 0, 0], 0, 10)], tg, med,
                               pp.Monochromatic(450.0), 1)
    t = pp.HitTable(wavelength=np.array([450.0, 500.0], np.float32),
                    dist_travelled=np.array([10.0, 40.0], np.float32),
                    base_weight=np.array([2.0, 2.0]))
    pp.calc_total_weight(t, setup)
    want = np.exp(-np.array([10.0 / 27.7, 40.0 / med.absorption_length(500.0)]))
    np.testing.assert_allclose(t["abs_weight"], want, rtol=1e-6)
    np.testing.assert_allclose(t["total_weight"], 2 * want, rtol=1e-6)


def test_workload_shapes(pp):
    s1 = pp.workloads.c1_setup(photons=10)
    assert len(s1.targets) == 400
    z = sorted({t.shape.position[2] for t in s1.targets})
    assert z[0] == -250.0 and z[-1] == 225.0 and len(z) == 20
    assert all(t.shape.radius == 0.2159 for t in s1.targets)
    p = s1.sources[0].position
    assert -250 <= p[2] <= 225
    s2 = pp.workloads.c2_setup()
    n = np.array([s.photons for s in s2.sources])
    assert len(n) == 256 and n.min() >= 1e4 and n.max() <= 1e7
    kinds = [s.kind for s in s2.sources]
    assert kinds.count(0) == 128 and kinds.count(1) == 128


def test_upload_record_follows_the_context(pp):
    """The device inputs a context holds are recorded on the context: a setup
    that another setup's upload replaced is uploaded again, equal derived
    tables count as the same, and a low-level setter clears the record."""
    import types
    m = pp.CascadiaMediumProperties()
    t = [pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 10.0], 0.3), 1.0, 1)]
    lp = pp.LongitudinalParameterisation(2.0, 0.63, 0.36)
    a = pp.PhotonPropSetup([pp.ExtendedCherenkovEmitter([0, 0, 0], [0, 0, 1.0], 0.0, 10, lp)], t,
                           m, pp.make_monochromatic_spectrum(450.0), 1)
    b = pp.PhotonPropSetup([pp.ExtendedCherenkovEmitterCustomSmear([0, 0, 0], [0, 0, 1.0], 0.0, 10,
                                                                   lp, 2.0, 0.5)], t, m,
                           pp.make_monochromatic_spectrum(450.0), 1)
    ctx = types.SimpleNamespace(uploaded=None)
    assert not a.is_uploaded(ctx)
    ctx.uploaded = a.upload_signature()
    assert a.is_uploaded(ctx)
    # same medium and targets, but another spectrum object and other smear tables
    assert not b.is_uploaded(ctx)
    ctx.uploaded = b.upload_signature()
    assert not a.is_uploaded(ctx)  # b's upload replaced a's inputs
    c = pp.PhotonPropSetup(list(a.sources), list(t), m, a.spec_dist, 2)
    ctx.uploaded = a.upload_signature()
    assert c.is_uploaded(ctx)  # same objects, another seed: nothing to send
    # new objects with equal values (another emitter position): nothing to send
    d = pp.PhotonPropSetup([pp.ExtendedCherenkovEmitter([5, 0, 0], [0, 0, 1.0], 0.0, 10, lp)],
                           [pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 10.0], 0.3), 1.0, 1)],
                           pp.CascadiaMediumProperties(), pp.make_monochromatic_spectrum(450.0), 3)
    assert d.is_uploaded(ctx)
    e = pp.PhotonPropSetup(list(a.sources),
                           [pp.HomogeneousDetector(pp.Spherical([0.0, 0.0, 10.5], 0.3), 1.0, 1)],
                           m, pp.make_monochromatic_spectrum(450.0), 1)
    assert not e.is_uploaded(ctx)  # a moved module must be sent
    assert not a.is_uploaded(types.SimpleNamespace(uploaded=None))
