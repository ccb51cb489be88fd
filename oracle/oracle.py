"""ctypes wrapper of the CPU ORACLE (oracle/pp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, never by the product.  Parity of the oracle
with PhotonPropagation.jl itself is unpinned (see pp_oracle.h).
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from ctypes import (POINTER, Structure, byref, c_double, c_float, c_int32, c_int64, c_uint32,
                    c_void_p)

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libpp_oracle.so")
SOURCES = [os.path.join(HERE, f) for f in ("pp_oracle.c", "pp_oracle_body.inc", "pp_oracle.h")]


def build(force: bool = False) -> str:
    """Compile the oracle with the host C compiler (portable flags only)."""
    deps = SOURCES + [os.path.join(os.path.dirname(HERE), "include", "pp_gb300.h")]
    if (not force and os.path.exists(LIB) and
            all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps)):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    cc = os.environ.get("CC") or shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11",
           "-shared", "-o", LIB + ".tmp", os.path.join(HERE, "pp_oracle.c"), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(LIB + ".tmp", LIB)
    return LIB


class ppo_medium(Structure):
    _fields_ = [
        ("kind", c_int32), ("n_abs", c_int32),
        ("hg_g", c_double), ("es_b", c_double), ("hg_weight", c_double),
        ("abs_scale", c_double), ("sca_scale", c_double),
        ("vol_conc_small", c_double), ("vol_conc_large", c_double),
        ("salinity", c_double), ("temperature", c_double), ("pressure", c_double),
        ("abs_wl", POINTER(c_double)), ("abs_len", POINTER(c_double)),
        ("s_sca_len", c_double), ("s_abs_len", c_double), ("s_ref_index", c_double),
        ("s_group_velocity", c_double),
        ("i_a_dust_400", c_double), ("i_b_dust_400", c_double), ("i_alpha_sca_dust", c_double),
        ("i_kappa_abs_dust", c_double), ("i_A", c_double), ("i_B", c_double),
        ("i_delta_t", c_double), ("i_mean_cos", c_double),
        ("phase_kind", c_int32), ("reserved_phase", c_int32),
    ]


class ppo_run(Structure):
    _fields_ = [
        ("sources", c_void_p), ("n_src", c_int32), ("photon_scaling", c_float),
        ("targets", c_void_p), ("n_targets", c_int32), ("n_steps", c_int32),
        ("medium", POINTER(ppo_medium)),
        ("spectrum_knots", POINTER(c_float)), ("n_spectrum", c_int32),
        ("mono_wavelength", c_float),
        ("track_quantiles", POINTER(c_float)), ("n_track", c_int32), ("reserved", c_int32),
        ("seed", c_int64), ("shapes", c_void_p), ("n_shapes", c_int32), ("reserved2", c_int32),
    ]


class ppo_stats(Structure):
    _fields_ = [("n_ph_sim", c_int64), ("photon_steps", c_int64), ("n_hits", c_int64)]


HIT_DTYPE = np.dtype([
    ("position", "<f8", (3,)), ("direction", "<f8", (3,)), ("initial_direction", "<f8", (3,)),
    ("wavelength", "<f8"), ("time", "<f8"), ("dist_travelled", "<f8"), ("abs_weight", "<f8"),
    ("photon_index", "<i8"), ("module_index", "<i4"), ("n_steps", "<i4"),
    ("source_index", "<i4"), ("reserved", "<i4"),
])

_L = None


def load():
    global _L
    if _L is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        fp = POINTER(c_float)
        dp = POINTER(c_double)
        L.ppo_philox4x32_10.argtypes = [POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]
        L.ppo_u01.restype = c_float
        L.ppo_u01.argtypes = [c_uint32]
        L.ppo_uniforms.argtypes = [c_int64, c_int32, c_int64, c_uint32, fp]
        L.ppo_source_photons.restype = c_int64
        L.ppo_source_photons.argtypes = [c_int64, c_float]
        L.ppo_medium_eval_f64.argtypes = [POINTER(ppo_medium), c_double, dp]
        L.ppo_medium_eval_f32.argtypes = [POINTER(ppo_medium), c_float, fp]
        L.ppo_dispersion_f64.restype = c_double
        L.ppo_dispersion_f64.argtypes = [POINTER(ppo_medium), c_double]
        for n, t in (("ppo_hg_cos_f64", c_double), ("ppo_es_cos_f64", c_double),
                     ("ppo_hg_cos_f32", c_float), ("ppo_es_cos_f32", c_float),
                     ("ppo_sl_cos_f64", c_double), ("ppo_sl_cos_f32", c_float)):
            getattr(L, n).restype = t
            getattr(L, n).argtypes = [t, t]
        L.ppo_rot_from_ez_f64.argtypes = [dp, dp, dp]
        L.ppo_rot_from_ez_f32.argtypes = [fp, fp, fp]
        L.ppo_spectrum_sample.restype = c_float
        L.ppo_spectrum_sample.argtypes = [fp, c_int32, c_float]
        L.ppo_quantile_sample.restype = c_float
        L.ppo_quantile_sample.argtypes = [fp, c_int32, c_float]
        L.ppo_gamma_f32.restype = c_float
        L.ppo_gamma_f32.argtypes = [c_int64, c_int32, c_int64, c_float, c_float, POINTER(c_uint32)]
        L.ppo_intersect_sphere_f32.restype = c_int32
        L.ppo_intersect_sphere_f32.argtypes = [fp, c_float, fp, fp, c_float, fp]
        L.ppo_init_photon_f32.restype = c_int32
        L.ppo_init_photon_f32.argtypes = [POINTER(ppo_run), c_int32, c_int64, fp, fp, fp, fp]
        for n in ("ppo_propagate_f32", "ppo_propagate_f64"):
            getattr(L, n).restype = c_int64
            getattr(L, n).argtypes = [POINTER(ppo_run), c_int32, c_int64, c_int64, c_void_p,
                                      c_int64, c_int32, POINTER(ppo_stats)]
        L.ppo_max_threads.restype = c_int32
        L.ppo_abi_layout.restype = c_int64
        L.ppo_abi_layout.argtypes = [ctypes.c_char_p]
        _L = L
    return _L


def philox(ctr, key) -> np.ndarray:
    L = load()
    c = (c_uint32 * 4)(*[int(x) & 0xffffffff for x in ctr])
    k = (c_uint32 * 2)(*[int(x) & 0xffffffff for x in key])
    o = (c_uint32 * 4)()
    L.ppo_philox4x32_10(c, k, o)
    return np.array(list(o), np.uint32)


def make_medium(params: dict):
    """ppo_medium from MediumProperties.oracle_params(); returns (struct, keepalive)."""
    m = ppo_medium()
    keep = []
    for k, v in params.items():
        if k in ("abs_wl", "abs_len"):
            a = np.ascontiguousarray(v, np.float64)
            keep.append(a)
            setattr(m, k, a.ctypes.data_as(POINTER(c_double)))
            m.n_abs = a.shape[0]
        else:
            setattr(m, k, v)
    return m, keep


class Run:
    """One oracle configuration: sources/targets as C-ABI records, the medium
    as analytic parameters, the same spectrum knots and track table as the
    device."""

    def __init__(self, source_records, n_src, sphere_records, n_targets, medium_params,
                 spectrum_knots=None, mono_wavelength=0.0, track_quantiles=None, seed=1,
                 n_steps=15, photon_scaling=1.0, shape_records=None):
        self.L = load()
        self._keep = [source_records, sphere_records]
        self.medium, k = make_medium(medium_params)
        self._keep += k
        r = ppo_run()
        r.sources = ctypes.cast(source_records, c_void_p)
        r.n_src = n_src
        r.photon_scaling = photon_scaling
        if shape_records is not None:
            self._keep.append(shape_records)
            r.shapes = ctypes.cast(shape_records, c_void_p)
            r.n_shapes = n_targets
            r.targets = None
            r.n_targets = 0
        else:
            r.targets = ctypes.cast(sphere_records, c_void_p) if n_targets else None
            r.n_targets = n_targets
        r.n_steps = n_steps
        r.medium = ctypes.pointer(self.medium)
        if spectrum_knots is not None:
            sk = np.ascontiguousarray(spectrum_knots, np.float32)
            self._keep.append(sk)
            r.spectrum_knots = sk.ctypes.data_as(POINTER(c_float))
            r.n_spectrum = sk.shape[0]
        r.mono_wavelength = mono_wavelength
        if track_quantiles is not None:
            tq = np.ascontiguousarray(track_quantiles, np.float32)
            self._keep.append(tq)
            r.track_quantiles = tq.ctypes.data_as(POINTER(c_float))
            r.n_track = tq.shape[-1]  # knots per table (tables stacked row-wise)
        r.seed = seed
        self.run = r

    @classmethod
    def from_setup(cls, setup, n_steps=15):
        shaped = setup.has_shaped_targets()
        return cls(setup.source_records(), len(setup.sources),
                   None if shaped else setup.sphere_records(),
                   setup.n_target_records(), setup.medium.oracle_params(),
                   shape_records=setup.target_records() if shaped else None,
                   spectrum_knots=setup.spectrum_knots,
                   mono_wavelength=setup.mono_wavelength or 0.0,
                   track_quantiles=setup.track_table_stack() if setup.needs_track_smear() else None,
                   seed=setup.seed, n_steps=n_steps, photon_scaling=setup.photon_scaling)

    def source_photons(self, src: int) -> int:
        s = ctypes.cast(self.run.sources, POINTER(ctypes.c_byte * 96))
        photons = int(np.frombuffer(bytes(s[src]), np.int64, 1, 8)[0])
        return self.L.ppo_source_photons(photons, self.run.photon_scaling)

    def propagate(self, src=0, begin=0, end=None, precision="f32", capacity=None, nthreads=0):
        if end is None:
            end = self.source_photons(src)
        cap = capacity if capacity is not None else max(1, end - begin)
        out = np.zeros(cap, HIT_DTYPE)
        st = ppo_stats()
        fn = self.L.ppo_propagate_f32 if precision == "f32" else self.L.ppo_propagate_f64
        n = fn(byref(self.run), src, begin, end, out.ctypes.data, cap, nthreads, byref(st))
        if n < 0:
            raise ValueError("oracle rejected its arguments")
        return out[:n], st

    def propagate_all(self, precision="f32", nthreads=0):
        hits, sim, steps = [], 0, 0
        for s in range(self.run.n_src):
            h, st = self.propagate(s, precision=precision, nthreads=nthreads)
            hits.append(h)
            sim += st.n_ph_sim
            steps += st.photon_steps
        return np.concatenate(hits) if hits else np.zeros(0, HIT_DTYPE), sim, steps
