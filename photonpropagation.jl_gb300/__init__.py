"""GB300-native photon transport behind PhotonPropagation.jl's API.

Host-side mirror of the reference's Julia interface for the photon-transport
hot path: ``PhotonPropSetup(sources, targets, medium, spectrum, seed)`` and
``propagate_photons(setup)``.  The propagation itself runs in the sm_103a CUDA
library ``_lib/libpp_gb300.so`` (C ABI in include/pp_gb300.h); there is no CPU
path.
"""
from . import _lib
from .context import Context, debug_philox, device_memory, measure_fp32_peak
from .medium import (C_VAC_M_NS, CascadiaMediumProperties, HomogenousIceProperties,
                     MediumProperties, SimpleMediumProperties, make_homogenous_clearice_properties)
from .processing import (HitBuffers, HitTable, PhotonPropOOMException, add_pmt_noise, autotune,
                         calc_number_of_steps, calc_total_weight, get_context, get_pmt_count,
                         make_hit_buffers, propagate_photons, resample_hits,
                         run_photon_prop_no_local_cache)
from .propsetup import PhotonPropSetup
from .sources import (AxiconeEmitter, CherenkovTrackEmitter, CollimatedIsotropicEmitter,
                      ExtendedCherenkovEmitter, ExtendedCherenkovEmitterCustomSmear,
                      ExtendedCherenkovEmitterNoSmear,
                      LongitudinalParameterisation, PencilEmitter, PointlikeCherenkovEmitter,
                      PointlikeIsotropicEmitter, PointlikeTimeRangeEmitter, source_photons)
from .spectrum import (InterpolatedSpectralDist, Monochromatic, Spectrum, frank_tamm,
                       make_biased_cherenkov_spectrum, make_cherenkov_spectrum, make_monochromatic_spectrum, make_spectral_dist)
from .targets import (Circular, DetectorLine, DetectorLines, HomogeneousDetector, Rectangular,
                      Spherical)
from . import calc, detection, dom, generic_multipmt, particles, pom, surrogate, workloads
from .particles import (Particle, cascade_cherenkov_track_length, particle_shape, propagate_particles,
                        rescale_source, split_source, total_lightyield)
from .calc import (calc_tgeo, calc_tgeo_tracks, calc_time_residual, closest_approach_distance,
                   closest_approach_param)
from .pom import POM
from .dom import DOM, DOMAcceptance
from .generic_multipmt import (SphericalMultiPMTTarget, fibonacci_sphere,
                               make_generic_multipmt_om, make_generic_multipmt_positions)
from .detection import (InterpQuantumEff, apply_qe, apply_wl_acceptance, calc_pe_weight,
                        check_pmt_hit, check_pmt_hit_opening_angle, make_hits_from_photons)

from .calc import (calc_time_residual_cascades, calc_time_residual_tracks, shift_particle,
                   shift_to_closest_approach)
from .particles import (AngularEmissionProfile, CherenkovTrackLengthParameters,
                        FastLightsabreMuonEmitter, LongitudinalParametersBase,
                        cherenkov_ang_dist, cherenkov_ang_dist_int, get_longitudinal_params)
from .pom import POMAcceptance, POMRelativeAcceptance, get_pom_pmt_group
from .processing import PhotonHit
from .sources import _CherenkovBase as CherenkovEmitter
from .spectrum import make_cuda_spectral_dist
from .targets import check_intersection
from . import output
from .output import (dataframe_to_hit_list, event_info_to_dataframe, hit_list_to_dataframe,
                     read_event, save_event, source_to_namedtuple, targets_to_dataframe)

__all__ = [n for n in dir() if not n.startswith("_")]

