"""PhotonPropSetup (mirrors src/photon_propagation_setup.jl:9-25)."""
from __future__ import annotations

import numpy as np

from . import sources as _sources
from . import targets as _targets
from .spectrum import InterpolatedSpectralDist, Monochromatic, SpectralDist, Spectrum

# Medium tables are sampled on a 0.125 nm grid: linear interpolation of the
# Kopelevich scattering length is then exact to about 2e-7 relative.
MEDIUM_TABLE_STEP_NM = 0.125


class PhotonPropSetup:
    """Sources, targets, medium, spectrum and seed of one propagation.

    ``PhotonPropSetup(sources, targets, medium, spectrum, seed;
    photon_scaling=1., spectrum_interp_steps=600)`` as in the reference.  The
    spectrum may be a ``Spectrum`` (as the reference requires) or, as in the
    reference README, a bare ``Monochromatic``/``InterpolatedSpectralDist``.
    ``track_smear`` optionally overrides the cos(theta) quantile table of the
    Cherenkov track direction.
    """

    def __init__(self, sources, targets, medium, spectrum, seed, photon_scaling=1.0,
                 spectrum_interp_steps=600, track_smear=None):
        self.sources = list(sources)
        self.targets = targets if isinstance(targets, _targets.DetectorLines) else list(targets)
        self.medium = medium
        if isinstance(spectrum, Spectrum):
            dist = spectrum.spectral_dist
        elif isinstance(spectrum, SpectralDist):
            dist = spectrum
        else:
            raise TypeError(f"unsupported spectrum {type(spectrum)}")
        self.spec_dist = dist
        if isinstance(dist, InterpolatedSpectralDist):
            self.spectrum_knots = dist.device_knots(spectrum_interp_steps)
            self.mono_wavelength = None
        elif isinstance(dist, Monochromatic):
            self.spectrum_knots = None
            self.mono_wavelength = float(np.float32(dist.wavelength))
        else:
            raise TypeError(f"unsupported spectral distribution {type(dist)}")
        self.seed = int(seed)
        self.photon_scaling = float(photon_scaling)
        self._track = None if track_smear is None else np.asarray(track_smear, np.float32)
        self._medium_tables = None  # derived device inputs, computed once
        self._signature = None

    # -- derived device inputs ------------------------------------------------
    def wavelength_range(self):
        if self.spectrum_knots is not None:
            return float(self.spectrum_knots.min()), float(self.spectrum_knots.max())
        return self.mono_wavelength, self.mono_wavelength

    def medium_tables(self):
        if self._medium_tables is None:
            lo, hi = self.wavelength_range()
            self._medium_tables = self.medium.tables(lo, hi, MEDIUM_TABLE_STEP_NM)
        return self._medium_tables

    def needs_track_smear(self) -> bool:
        return any(s.kind in _sources.TRACK_SMEAR_KINDS for s in self.sources)

    def track_quantiles(self):
        if self._track is None:
            from .track_smear import beta_track_quantiles
            self._track = beta_track_quantiles()
        return self._track

    def _smear_tables(self):
        """cos(theta) quantile tables of the track smear: table 0 serves the
        Cherenkov emitters (the default Beta or the `track_smear` override),
        then one per distinct Beta(a, b) of ExtendedCherenkovEmitterCustomSmear
        sources; and the table index of every source."""
        from .track_smear import beta_track_quantiles
        tables = [np.asarray(self.track_quantiles(), np.float32)]
        keys = {}
        index = []
        for s in self.sources:
            if isinstance(s, _sources.ExtendedCherenkovEmitterCustomSmear):
                key = (float(s.cherenkov_beta_a), float(s.cherenkov_beta_b))
                if key not in keys:
                    q = beta_track_quantiles(*key, n=len(tables[0]))
                    if np.array_equal(q, tables[0]):
                        keys[key] = 0
                    else:
                        keys[key] = len(tables)
                        tables.append(q)
                index.append(keys[key])
            else:
                index.append(0)
        return np.stack(tables), index

    def track_table_stack(self) -> np.ndarray:
        """(n_tables, n_knots) float32 quantile tables for pp_set_track_smear_tables."""
        return self._smear_tables()[0]

    def source_records(self):
        recs = _sources.to_records(self.sources)
        if self.needs_track_smear():
            for i, t in enumerate(self._smear_tables()[1]):
                recs[i].smear_table = t
        return recs

    def sphere_records(self):
        return _targets.to_spheres(self.targets)

    def has_shaped_targets(self) -> bool:
        return _targets.is_shaped(self.targets)

    def target_records(self):
        return _targets.to_targets(self.targets)

    def n_target_records(self) -> int:
        return _targets.record_count(self.targets)

    def upload(self, ctx, cell_size: float = 0.0) -> None:
        """Send medium, spectrum, track table and targets to a Context."""
        ctx.set_medium(self.medium_tables())
        if self.spectrum_knots is not None:
            ctx.set_spectrum(self.spectrum_knots)
        else:
            ctx.set_monochromatic(self.mono_wavelength)
        if self.needs_track_smear():
            ctx.set_track_smear_tables(self.track_table_stack())
        if self.has_shaped_targets():
            ctx.set_shaped_targets(self.target_records(), self.n_target_records())
        else:
            ctx.set_targets(self.sphere_records(), len(self.targets), cell_size)
        ctx.uploaded = self.upload_signature(cell_size)

    def upload_signature(self, cell_size: float = 0.0):
        """What `upload` sends, by value: the medium tables and phase function,
        the spectrum knots (or wavelength), the track tables and the target
        records as bytes, plus the grid cell size.  Two setups with the same
        detector and medium (say, one per emitter position) then share one
        upload, as the reference's setups share nothing but upload once each.
        Computed once per setup: media, spectra and targets are taken as
        immutable once used, as the reference's structs are."""
        if self._signature is None:
            t = self.medium_tables()
            med = (float(t.wl_min), float(t.wl_step), t.scattering_length.tobytes(),
                   t.group_velocity.tobytes(), t.absorption_length.tobytes(),
                   t.phase_refractive_index.tobytes(), float(t.hg_g), float(t.es_b),
                   float(t.hg_weight), int(t.phase_kind))
            shaped = self.has_shaped_targets()
            recs = self.target_records() if shaped else self.sphere_records()
            knots = None if self.spectrum_knots is None else \
                np.asarray(self.spectrum_knots, np.float32).tobytes()
            tables = self.track_table_stack().tobytes() if self.needs_track_smear() else None
            self._signature = (med, shaped, bytes(memoryview(recs).cast("B")), knots,
                               self.mono_wavelength, tables)
        return self._signature + (float(cell_size),)

    def is_uploaded(self, ctx, cell_size: float = 0.0) -> bool:
        """True when `ctx` holds exactly what `upload` would send."""
        return getattr(ctx, "uploaded", None) == self.upload_signature(cell_size)
