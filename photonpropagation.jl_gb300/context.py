"""Python handle on a pp_ctx (one device, its tables, its work queue).

Thin, allocation-aware wrapper over the C ABI; used by the reference-shaped
API in ``processing`` and directly by benchmarks that keep buffers on the
device.
"""
from __future__ import annotations

import ctypes
from ctypes import byref, c_double, c_float, c_int32, c_int64, c_uint32, c_void_p

import numpy as np

from . import _lib
from ._lib import PPError, check

HIT_COLUMNS = {
    # name: (dtype, trailing shape)
    "position": (np.float32, (3,)),
    "direction": (np.float32, (3,)),
    "initial_direction": (np.float32, (3,)),
    "wavelength": (np.float32, ()),
    "time": (np.float64, ()),
    "dist_travelled": (np.float32, ()),
    "abs_weight": (np.float32, ()),
    "module_index": (np.int32, ()),
    "n_steps": (np.int32, ()),
    "source_index": (np.int32, ()),
    "photon_index": (np.int64, ()),
}


def alloc_columns(n: int) -> dict:
    return {k: np.empty((n,) + shp, dt) for k, (dt, shp) in HIT_COLUMNS.items()}


def columns_struct(cols: dict) -> _lib.pp_hits:
    h = _lib.pp_hits()
    for k in HIT_COLUMNS:
        a = cols.get(k)
        if a is None:
            continue
        if isinstance(a, int):  # raw device pointer
            setattr(h, k, a)
        else:
            assert a.flags["C_CONTIGUOUS"]
            setattr(h, k, a.ctypes.data)
    return h


def device_memory(device: int = 0):
    lib = _lib.load()
    f, t = c_int64(), c_int64()
    check(lib.pp_device_memory(device, byref(f), byref(t)), "pp_device_memory")
    return f.value, t.value


def measure_fp32_peak(device: int = 0) -> float:
    lib = _lib.load()
    v = c_double()
    check(lib.pp_measure_fp32_peak(device, byref(v)), "pp_measure_fp32_peak")
    return v.value


def debug_philox(ctr: np.ndarray, key0: int, key1: int) -> np.ndarray:
    lib = _lib.load()
    ctr = np.ascontiguousarray(ctr, np.uint32).reshape(-1, 4)
    out = np.empty_like(ctr)
    check(lib.pp_debug_philox(ctr.ctypes.data_as(ctypes.POINTER(c_uint32)), ctr.shape[0],
                              key0, key1, out.ctypes.data_as(ctypes.POINTER(c_uint32))),
          "pp_debug_philox")
    return out


class Context:
    def __init__(self, device: int = 0):
        self._lib = _lib.load()
        p = c_void_p()
        check(self._lib.pp_create(byref(p), device), "pp_create")
        self.ptr = p
        self.device = device
        self._keep = {}
        self.uploaded = None  # what the last PhotonPropSetup.upload sent

    def close(self):
        if getattr(self, "ptr", None) and self.ptr.value:
            self._lib.pp_destroy(self.ptr)
            self.ptr = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- tables -------------------------------------------------------------
    def set_medium(self, t) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        arrs = [np.ascontiguousarray(a, np.float32) for a in
                (t.scattering_length, t.group_velocity, t.absorption_length,
                 t.phase_refractive_index)]
        m = _lib.pp_medium()
        m.wl_min, m.wl_step, m.n_knots = t.wl_min, t.wl_step, arrs[0].shape[0]
        fp = ctypes.POINTER(c_float)
        m.scattering_length = arrs[0].ctypes.data_as(fp)
        m.group_velocity = arrs[1].ctypes.data_as(fp)
        m.absorption_length = arrs[2].ctypes.data_as(fp)
        m.phase_refractive_index = arrs[3].ctypes.data_as(fp)
        m.hg_g, m.es_b, m.hg_weight = t.hg_g, t.es_b, t.hg_weight
        m.phase_kind = int(getattr(t, "phase_kind", 0))
        check(self._lib.pp_set_medium(self.ptr, byref(m)), "pp_set_medium")

    def set_spectrum(self, knots) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        k = np.ascontiguousarray(knots, np.float32)
        check(self._lib.pp_set_spectrum(self.ptr, k.ctypes.data_as(ctypes.POINTER(c_float)),
                                        k.shape[0]), "pp_set_spectrum")

    def set_monochromatic(self, wl: float) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        check(self._lib.pp_set_monochromatic(self.ptr, float(wl)), "pp_set_monochromatic")

    def set_track_smear(self, q) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        q = np.ascontiguousarray(q, np.float32)
        check(self._lib.pp_set_track_smear(self.ptr, q.ctypes.data_as(ctypes.POINTER(c_float)),
                                           q.shape[0]), "pp_set_track_smear")

    def set_track_smear_tables(self, q) -> None:
        """(n_tables, n_knots) quantile tables; a source uses its smear_table."""
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        q = np.ascontiguousarray(np.atleast_2d(q), np.float32)
        check(self._lib.pp_set_track_smear_tables(
            self.ptr, q.ctypes.data_as(ctypes.POINTER(c_float)), q.shape[1], q.shape[0]),
            "pp_set_track_smear_tables")

    def set_targets(self, spheres, n: int, cell_size: float = 0.0) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        check(self._lib.pp_set_targets(self.ptr, spheres, n, float(cell_size)), "pp_set_targets")

    def set_shaped_targets(self, records, n: int) -> None:
        self.uploaded = None  # device inputs changed outside PhotonPropSetup.upload
        check(self._lib.pp_set_shaped_targets(self.ptr, records, n), "pp_set_shaped_targets")

    def set_sources(self, records, n: int, scaling: float = 1.0) -> None:
        check(self._lib.pp_set_sources(self.ptr, records, n, float(scaling)), "pp_set_sources")

    def total_photons(self) -> int:
        v = c_int64()
        check(self._lib.pp_total_photons(self.ptr, byref(v)))
        return v.value

    # -- tuning -------------------------------------------------------------------
    def get_tuning(self) -> _lib.pp_tuning:
        t = _lib.pp_tuning()
        check(self._lib.pp_get_tuning(self.ptr, byref(t)))
        return t

    def set_tuning(self, **kw) -> _lib.pp_tuning:
        t = self.get_tuning()
        for k, v in kw.items():
            setattr(t, k, v)
        check(self._lib.pp_set_tuning(self.ptr, byref(t)), "pp_set_tuning")
        return t

    def autotune(self, seed: int, n_steps: int, sample_photons: int = 4_000_000):
        t = _lib.pp_tuning()
        rate = c_double()
        check(self._lib.pp_autotune(self.ptr, seed, n_steps, sample_photons, byref(t),
                                    byref(rate)), "pp_autotune")
        return t, rate.value

    def grid_info(self) -> dict:
        dims = (c_int32 * 3)()
        cell = (c_float * 3)()
        org = (c_float * 3)()
        ni, nb = c_int64(), c_int64()
        check(self._lib.pp_grid_info(self.ptr, dims, cell, org, byref(ni), byref(nb)))
        return dict(dims=tuple(dims), cell=tuple(cell), origin=tuple(org), n_items=ni.value,
                    blob_bytes=nb.value)

    # -- running --------------------------------------------------------------------
    def launch(self, seed: int, n_steps: int, d_hits: int, capacity: int, d_counters: int,
               stream: int = 0, graph: bool = False) -> None:
        fn = self._lib.pp_launch_graph if graph else self._lib.pp_launch
        check(fn(self.ptr, seed, n_steps, c_void_p(d_hits), capacity, c_void_p(d_counters),
                 c_void_p(stream)), "pp_launch_graph" if graph else "pp_launch")

    def propagate(self, records, n: int, seed: int, n_steps: int, scaling: float,
                  capacity: int):
        """Synchronous propagate into context-owned buffers.  Returns
        (status, n_hits, n_ph_sim); status is PP_OK or PP_ERR_OVERFLOW."""
        nh, ns = c_int64(), c_int64()
        rc = self._lib.pp_propagate(self.ptr, records, n, seed, n_steps, float(scaling), None,
                                    capacity, byref(nh), byref(ns))
        check(rc, "pp_propagate")
        return rc, nh.value, ns.value

    def fetch_hits(self, n: int, cols: dict | None = None) -> dict:
        cols = alloc_columns(n) if cols is None else cols
        if n > 0:
            h = columns_struct(cols)
            check(self._lib.pp_fetch_hits(self.ptr, byref(h), n), "pp_fetch_hits")
        return cols
