/*
 * pp_oracle.h -- CPU ORACLE for the photon-transport hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of
 * PhotonPropagation.jl v0.9.3's per-photon step functions, used by the test
 * suite, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
 * checker.  The product (the CUDA library and its Python/Julia host side)
 * never links, loads or calls it.
 *
 * Parity status: UNPINNED against the reference itself.  The reference is
 * Julia + CUDA.jl and cannot run in this build environment, its own tests do
 * not touch this path (test/test_calc.jl only checks closest_approach_distance)
 * and it ships no golden vectors.  Part of the arithmetic lives in packages
 * absent from the reference tree, restated here from their published
 * algorithms:
 *   CherenkovMediumBase 1.0.0 (Manifest.toml:217-221): Kopelevich scattering
 *     length, Quan & Fry (1995) refractive index with a linear pressure term,
 *     group velocity, Henyey-Greenstein and Einstein-Smoluchowski phase
 *     functions mixed as MixedHGES(g, b, w) with w = P(HG), linear
 *     interpolation of the absorption table, Cherenkov angle acos(1/n).
 *   PhysicsTools 0.8.2 (Manifest.toml:911-915): sph_to_cart, rotation taking
 *     e_z onto a vector (rot_from_ez_fast), Marsaglia-Tsang gamma sampling.
 *   CUDA.jl 5.6.1 device RNG: replaced by Philox4x32-10 (Salmon et al.,
 *     SC'11) keyed on (seed) and counted on (photon, call, source).
 * The oracle is pinned instead by: Philox known-answer vectors, analytic
 * known-answer tests (exponential step mean, HG mean cosine, ES moments,
 * isotropy, unscattered hit fraction, Frank-Tamm CDF) and the reference's own
 * absorption-length table (assets/attenuation_length_straw_fit.parquet).
 *
 * Built twice from one body: *_f32 computes in FP32 as the reference kernel
 * does (time accumulated step by step in FP32, src/photon_prop_cuda.jl:511,519),
 * *_f64 computes everything in FP64 on the same random numbers.
 */
#ifndef PP_ORACLE_H
#define PP_ORACLE_H

#include <stdint.h>

#include "../include/pp_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Medium description evaluated analytically (per photon, like
 * scattering_length / group_velocity at src/photon_prop_cuda.jl:480-482). */
#define PPO_MEDIUM_CASCADIA 0 /* src/water_properties.jl:43-100 */
#define PPO_MEDIUM_SIMPLE 1   /* src/simple_medium.jl:1-15      */
#define PPO_MEDIUM_ICE 2      /* src/ice_properties.jl:26-176   */

typedef struct ppo_medium {
  int32_t kind;
  int32_t n_abs;             /* absorption table length (Cascadia)          */
  double hg_g, es_b, hg_weight;
  double abs_scale, sca_scale;
  double vol_conc_small, vol_conc_large; /* Kopelevich (ppm)               */
  double salinity, temperature, pressure; /* Quan & Fry: permille, C, atm  */
  const double* abs_wl;      /* nm                                          */
  const double* abs_len;     /* m                                           */
  /* SIMPLE medium constants */
  double s_sca_len, s_abs_len, s_ref_index, s_group_velocity;
  /* ICE (HomogenousIceProperties): SPICE dust coefficients at 400 nm and
   * exponents, the A/B/delta-T pure-ice absorption terms, mean cos */
  double i_a_dust_400, i_b_dust_400, i_alpha_sca_dust, i_kappa_abs_dust;
  double i_A, i_B, i_delta_t, i_mean_cos;
  int32_t phase_kind; /* PP_PHASE_HG_ES or PP_PHASE_HG_SL */
  int32_t reserved_phase;
} ppo_medium;

/* One oracle hit (all fields widened to double). */
typedef struct ppo_hit {
  double position[3];
  double direction[3];
  double initial_direction[3];
  double wavelength;
  double time;
  double dist_travelled;
  double abs_weight;
  int64_t photon_index;
  int32_t module_index; /* 1-based */
  int32_t n_steps;
  int32_t source_index;
  int32_t reserved;
} ppo_hit;

typedef struct ppo_run {
  const pp_source* sources;
  int32_t n_src;
  float photon_scaling;
  const pp_sphere* targets;
  int32_t n_targets;
  int32_t n_steps;
  const ppo_medium* medium;
  const float* spectrum_knots; /* inverse CDF knots; NULL => monochromatic */
  int32_t n_spectrum;
  float mono_wavelength;
  const float* track_quantiles; /* cos(theta) quantiles of the track smear */
  int32_t n_track;
  int32_t reserved;
  int64_t seed;
  /* shaped targets (used instead of `targets` when n_shapes > 0): spheres,
   * rectangles and discs tested in index order (check_intersection,
   * src/photon_prop_cuda.jl:345-404) */
  const pp_target* shapes;
  int32_t n_shapes;
  int32_t reserved2;
} ppo_run;

typedef struct ppo_stats {
  int64_t n_ph_sim;
  int64_t photon_steps;
  int64_t n_hits;  /* hits found (may exceed capacity) */
} ppo_stats;

/* Philox4x32-10: out = bijection(ctr) under key. */
void ppo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* 24-bit uniform in (0, 1]. */
float ppo_u01(uint32_t x);
/* The four uniforms of call `call` of photon `photon` of source `src`. */
void ppo_uniforms(int64_t seed, int32_t src, int64_t photon, uint32_t call, float u[4]);

/* Photon count of a source: floor(Float32(photons) * scaling) in FP32
 * (src/photon_prop_cuda.jl:456). */
int64_t ppo_source_photons(int64_t photons, float scaling);

/* Medium at `wl` (nm): out = {scattering_length, group_velocity,
 * absorption_length, phase_refractive_index}. */
void ppo_medium_eval_f64(const ppo_medium* m, double wl, double out[4]);
void ppo_medium_eval_f32(const ppo_medium* m, float wl, float out[4]);
double ppo_dispersion_f64(const ppo_medium* m, double wl); /* dn/dlambda, 1/nm */

/* Phase functions on one uniform. */
double ppo_hg_cos_f64(double g, double eta);
float ppo_hg_cos_f32(float g, float eta);
double ppo_es_cos_f64(double b, double eta);
float ppo_es_cos_f32(float b, float eta);
/* Simplified Liu, p(x) ~ (1 + x)^(2g/(1-g)): x = 2 eta^((1-g)/(1+g)) - 1. */
double ppo_sl_cos_f64(double g, double eta);
float ppo_sl_cos_f32(float g, float eta);

/* Rotation taking e_z onto unit vector a, applied to b. */
void ppo_rot_from_ez_f64(const double a[3], const double b[3], double out[3]);
void ppo_rot_from_ez_f32(const float a[3], const float b[3], float out[3]);

/* Wavelength from the inverse-CDF knots as a linear-filtered, clamped texture
 * with normalised coordinates (src/spectrum.jl:79-83, :137-138). */
float ppo_spectrum_sample(const float* knots, int32_t n, float u);

/* Quantile-table lookup (knots at u = i/(n-1)). */
float ppo_quantile_sample(const float* q, int32_t n, float u);

/* Gamma(shape, scale) from the extra-draw stream of one photon. */
float ppo_gamma_f32(int64_t seed, int32_t src, int64_t photon, float shape, float scale,
                    uint32_t* calls_used);

/* Ray-sphere test of src/photon_prop_cuda.jl:309-343; returns 1 on a hit and
 * writes the distance. */
int ppo_intersect_sphere_f32(const float c[3], float rsq, const float pos[3], const float dir[3],
                             float step, float* d);

/* Initial photon state (position, direction, time, wavelength) of photon
 * `photon` of source `src` (initialize_photon_state, src/photon_prop_cuda.jl:158-276).
 * Returns 0 or -1 on unknown kind. */
int ppo_init_photon_f32(const ppo_run* run, int32_t src, int64_t photon, float pos[3],
                        float dir[3], float* time, float* wl);

/* Propagate photons [begin, end) of source `src` (local indices, clipped to
 * the source's photon count; the global photon index, which keys the random
 * numbers, is first_photon + local index), brute-force target loop in index order, first
 * intersected target wins (src/photon_prop_cuda.jl:466-543).  Appends up to
 * `capacity` hits to out (in no particular order when nthreads > 1) and
 * returns the number written, or -1 on bad arguments.  nthreads <= 0 uses all
 * OpenMP threads. */
int64_t ppo_propagate_f32(const ppo_run* run, int32_t src, int64_t begin, int64_t end,
                          ppo_hit* out, int64_t capacity, int32_t nthreads, ppo_stats* stats);
int64_t ppo_propagate_f64(const ppo_run* run, int32_t src, int64_t begin, int64_t end,
                          ppo_hit* out, int64_t capacity, int32_t nthreads, ppo_stats* stats);

/* Number of OpenMP threads available. */
int32_t ppo_max_threads(void);

/* sizeof and selected field offsets of the C-ABI structs as this C compiler
 * lays them out from include/pp_gb300.h (checked against the ctypes mirror);
 * -1 for an unknown name. */
int64_t ppo_abi_layout(const char* what);

#ifdef __cplusplus
}
#endif

#endif /* PP_ORACLE_H */
