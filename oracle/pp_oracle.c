/*
 * pp_oracle.c -- CPU ORACLE (test infrastructure only; see pp_oracle.h).
 *
 * Restates PhotonPropagation.jl v0.9.3's photon-transport step functions in
 * plain C.  Every function cites the reference file:line it follows (paths
 * inside the reference project).  Parity with the reference is UNPINNED
 * (see pp_oracle.h for why and for what pins the oracle instead).
 */
#include "pp_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------- Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) ------- */

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

static void philox_round(uint32_t c[4], const uint32_t k[2]) {
  uint64_t p0 = (uint64_t)PHILOX_M0 * (uint64_t)c[0];
  uint64_t p1 = (uint64_t)PHILOX_M1 * (uint64_t)c[2];
  uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
  uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
  uint32_t n0 = hi1 ^ c[1] ^ k[0];
  uint32_t n2 = hi0 ^ c[3] ^ k[1];
  c[0] = n0;
  c[1] = lo1;
  c[2] = n2;
  c[3] = lo0;
}

void ppo_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  uint32_t k[2] = {key[0], key[1]};
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k[0] += PHILOX_W0;
      k[1] += PHILOX_W1;
    }
    philox_round(c, k);
  }
  memcpy(out, c, sizeof(c));
}

float ppo_u01(uint32_t x) { return (float)((x >> 8) + 1u) * (1.0f / 16777216.0f); }

/* Counter layout: (photon low word, photon high word, call, source);
 * key: (seed low word, seed high word). */
void ppo_uniforms(int64_t seed, int32_t src, int64_t photon, uint32_t call, float u[4]) {
  uint32_t ctr[4] = {(uint32_t)((uint64_t)photon & 0xffffffffu), (uint32_t)((uint64_t)photon >> 32),
                     call, (uint32_t)src};
  uint32_t key[2] = {(uint32_t)((uint64_t)seed & 0xffffffffu), (uint32_t)((uint64_t)seed >> 32)};
  uint32_t r[4];
  ppo_philox4x32_10(ctr, key, r);
  for (int i = 0; i < 4; ++i) u[i] = ppo_u01(r[i]);
}

#define PPO_EXTRA_CALL 0x80000000u
#define PPO_GAMMA_MAX_TRIES 64

/* src/photon_prop_cuda.jl:456 -- Int64 * Float32 promotes to Float32. */
int64_t ppo_source_photons(int64_t photons, float scaling) {
  float x = (float)photons * scaling;
  if (!(x > 0.0f)) return 0;
  return (int64_t)floorf(x);
}

/* ---------------- medium (src/water_properties.jl:43-100) ----------------- */

static const double C_VAC_M_NS = 0.299792458;

/* Kopelevich scattering coefficient (1/m) at wl (nm): pure water + small and
 * large particles with volume concentrations in ppm. */
static double kopelevich_coeff_f64(const ppo_medium* m, double wl) {
  double x = 550.0 / wl;
  return 0.0017 * pow(x, 4.3) + 1.34 * m->vol_conc_small * pow(x, 1.7) +
         0.312 * m->vol_conc_large * pow(x, 0.3);
}
static float kopelevich_coeff_f32(const ppo_medium* m, float wl) {
  float x = 550.0f / wl;
  return 0.0017f * powf(x, 4.3f) + 1.34f * (float)m->vol_conc_small * powf(x, 1.7f) +
         0.312f * (float)m->vol_conc_large * powf(x, 0.3f);
}

/* Quan & Fry (1995) phase refractive index of sea water, wl in nm, S in
 * permille, T in C, plus a linear pressure term of 1.45e-5 per atm. */
static double quan_fry_f64(const ppo_medium* m, double wl) {
  double S = m->salinity, T = m->temperature, P = m->pressure;
  double x = 1.0 / wl;
  return 1.31405 + 1.45e-5 * P + (1.779e-4 - 1.05e-6 * T + 1.6e-8 * T * T) * S - 2.02e-6 * T * T +
         (15.868 + 0.01155 * S - 0.00423 * T) * x - 4382.0 * x * x + 1.1455e6 * x * x * x;
}
static float quan_fry_f32(const ppo_medium* m, float wl) {
  float S = (float)m->salinity, T = (float)m->temperature, P = (float)m->pressure;
  float x = 1.0f / wl;
  return 1.31405f + 1.45e-5f * P + (1.779e-4f - 1.05e-6f * T + 1.6e-8f * T * T) * S -
         2.02e-6f * T * T + (15.868f + 0.01155f * S - 0.00423f * T) * x - 4382.0f * x * x +
         1.1455e6f * x * x * x;
}
double ppo_dispersion_f64(const ppo_medium* m, double wl) {
  if (m->kind == PPO_MEDIUM_SIMPLE) return 0.0;
  double S = m->salinity, T = m->temperature;
  double x = 1.0 / wl;
  return -(15.868 + 0.01155 * S - 0.00423 * T) * x * x + 2.0 * 4382.0 * x * x * x -
         3.0 * 1.1455e6 * x * x * x * x;
}
static float dispersion_f32(const ppo_medium* m, float wl) {
  float S = (float)m->salinity, T = (float)m->temperature;
  float x = 1.0f / wl;
  return -(15.868f + 0.01155f * S - 0.00423f * T) * x * x + 2.0f * 4382.0f * x * x * x -
         3.0f * 1.1455e6f * x * x * x * x;
}

static double abs_interp_f64(const ppo_medium* m, double wl) {
  int n = m->n_abs;
  if (n <= 0) return INFINITY;
  if (wl <= m->abs_wl[0]) return m->abs_len[0];
  if (wl >= m->abs_wl[n - 1]) return m->abs_len[n - 1];
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (m->abs_wl[mid] <= wl) lo = mid; else hi = mid;
  }
  double f = (wl - m->abs_wl[lo]) / (m->abs_wl[hi] - m->abs_wl[lo]);
  return m->abs_len[lo] + f * (m->abs_len[hi] - m->abs_len[lo]);
}

/* Deep ice (src/ice_properties.jl:108-176): phase index polynomial in
 * wl/1000, group index = n times a second polynomial, absorption = SPICE dust
 * a_dust (wl/400)^-kappa plus A exp(-B/wl) (1 + 0.01 dT), scattering =
 * b_dust (wl/400)^-alpha / (1 - <cos>). */
static void ice_eval_f64(const ppo_medium* m, double wl, double out[4]) {
  double x = wl / 1000.0;
  double n = 1.55749 - 1.57988 * x + 3.99993 * x * x - 4.68271 * x * x * x +
             2.09354 * x * x * x * x;
  double ng = n * (1.0 + 0.227106 - 0.954648 * x + 1.42568 * x * x - 0.711832 * x * x * x);
  double a = m->i_a_dust_400 * pow(wl / 400.0, -m->i_kappa_abs_dust) +
             m->i_A * exp(-m->i_B / wl) * (1.0 + 0.01 * m->i_delta_t);
  double b = m->i_b_dust_400 * pow(wl / 400.0, -m->i_alpha_sca_dust) / (1.0 - m->i_mean_cos);
  out[0] = 1.0 / b * m->sca_scale;
  out[1] = C_VAC_M_NS / ng;
  out[2] = 1.0 / a * m->abs_scale;
  out[3] = n;
}
static void ice_eval_f32(const ppo_medium* m, float wl, float out[4]) {
  float x = wl / 1000.0f;
  float n = 1.55749f - 1.57988f * x + 3.99993f * x * x - 4.68271f * x * x * x +
            2.09354f * x * x * x * x;
  float ng = n * (1.0f + 0.227106f - 0.954648f * x + 1.42568f * x * x - 0.711832f * x * x * x);
  float a = (float)m->i_a_dust_400 * powf(wl / 400.0f, -(float)m->i_kappa_abs_dust) +
            (float)m->i_A * expf(-(float)m->i_B / wl) * (1.0f + 0.01f * (float)m->i_delta_t);
  float b = (float)m->i_b_dust_400 * powf(wl / 400.0f, -(float)m->i_alpha_sca_dust) /
            (1.0f - (float)m->i_mean_cos);
  out[0] = 1.0f / b * (float)m->sca_scale;
  out[1] = (float)C_VAC_M_NS / ng;
  out[2] = 1.0f / a * (float)m->abs_scale;
  out[3] = n;
}

void ppo_medium_eval_f64(const ppo_medium* m, double wl, double out[4]) {
  if (m->kind == PPO_MEDIUM_ICE) {
    ice_eval_f64(m, wl, out);
    return;
  }
  if (m->kind == PPO_MEDIUM_SIMPLE) { /* src/simple_medium.jl:11-15 */
    out[0] = m->s_sca_len;
    out[1] = m->s_group_velocity;
    out[2] = m->s_abs_len;
    out[3] = m->s_ref_index;
    return;
  }
  double n = quan_fry_f64(m, wl);
  double lam0 = n * wl; /* group index n - (n*wl) * dn/dwl */
  double ng = n - lam0 * ppo_dispersion_f64(m, wl);
  out[0] = 1.0 / kopelevich_coeff_f64(m, wl) * m->sca_scale; /* :95-100 */
  out[1] = C_VAC_M_NS / ng;
  out[2] = abs_interp_f64(m, wl) * m->abs_scale; /* :88-93 */
  out[3] = n;
}

void ppo_medium_eval_f32(const ppo_medium* m, float wl, float out[4]) {
  if (m->kind == PPO_MEDIUM_ICE) {
    ice_eval_f32(m, wl, out);
    return;
  }
  if (m->kind == PPO_MEDIUM_SIMPLE) {
    out[0] = (float)m->s_sca_len;
    out[1] = (float)m->s_group_velocity;
    out[2] = (float)m->s_abs_len;
    out[3] = (float)m->s_ref_index;
    return;
  }
  float n = quan_fry_f32(m, wl);
  float lam0 = n * wl;
  float ng = n - lam0 * dispersion_f32(m, wl);
  out[0] = 1.0f / kopelevich_coeff_f32(m, wl) * (float)m->sca_scale;
  out[1] = (float)C_VAC_M_NS / ng;
  out[2] = (float)abs_interp_f64(m, (double)wl) * (float)m->abs_scale;
  out[3] = n;
}

/* ---------------- phase functions (CherenkovMediumBase) ------------------- */

/* Henyey-Greenstein inverse CDF, clamped to [-1, 1]. */
double ppo_hg_cos_f64(double g, double eta) {
  double t = (1.0 - g * g) / (1.0 + g * (2.0 * eta - 1.0));
  double c = 1.0 / (2.0 * g) * (1.0 + g * g - t * t);
  return c < -1.0 ? -1.0 : (c > 1.0 ? 1.0 : c);
}
float ppo_hg_cos_f32(float g, float eta) {
  float t = (1.0f - g * g) / (1.0f + g * (2.0f * eta - 1.0f));
  float c = 1.0f / (2.0f * g) * (1.0f + g * g - t * t);
  return c < -1.0f ? -1.0f : (c > 1.0f ? 1.0f : c);
}

/* Einstein-Smoluchowski p(x) ~ 1 + b x^2: Cardano root of
 * x^3 + (3/b) x - (3+b)(2 eta - 1)/b = 0. */
double ppo_es_cos_f64(double b, double eta) {
  double q = (b + 3.0) * (eta - 0.5) / b;
  double d = sqrt(q * q + 1.0 / (b * b * b));
  return cbrt(q + d) + cbrt(q - d);
}
float ppo_es_cos_f32(float b, float eta) {
  float q = (b + 3.0f) * (eta - 0.5f) / b;
  float d = sqrtf(q * q + 1.0f / (b * b * b));
  return cbrtf(q + d) + cbrtf(q - d);
}

/* Simplified Liu inverse CDF (the SL half of mixed_hg_sl_scattering_func_ppc,
 * CherenkovMediumBase 1.0.0, as PPC samples it). */
double ppo_sl_cos_f64(double g, double eta) {
  return 2.0 * pow(eta, (1.0 - g) / (1.0 + g)) - 1.0;
}
float ppo_sl_cos_f32(float g, float eta) {
  return 2.0f * powf(eta, (1.0f - g) / (1.0f + g)) - 1.0f;
}

/* ---------------- geometry (PhysicsTools) ---------------------------------- */

void ppo_rot_from_ez_f64(const double a[3], const double b[3], double out[3]) {
  double s2 = a[0] * a[0] + a[1] * a[1];
  if (s2 == 0.0) {
    double sg = a[2] >= 0.0 ? 1.0 : -1.0;
    out[0] = sg * b[0]; out[1] = sg * b[1]; out[2] = sg * b[2];
    return;
  }
  double f = a[2] >= 0.0 ? 1.0 / (1.0 + a[2]) : (1.0 - a[2]) / s2;
  double k = (a[0] * b[1] - a[1] * b[0]) * f;
  out[0] = b[0] * a[2] + a[0] * b[2] - a[1] * k;
  out[1] = b[1] * a[2] + a[1] * b[2] + a[0] * k;
  out[2] = b[2] * a[2] - (a[0] * b[0] + a[1] * b[1]);
}
void ppo_rot_from_ez_f32(const float a[3], const float b[3], float out[3]) {
  float s2 = a[0] * a[0] + a[1] * a[1];
  if (s2 == 0.0f) {
    float sg = a[2] >= 0.0f ? 1.0f : -1.0f;
    out[0] = sg * b[0]; out[1] = sg * b[1]; out[2] = sg * b[2];
    return;
  }
  float f = a[2] >= 0.0f ? 1.0f / (1.0f + a[2]) : (1.0f - a[2]) / s2;
  float k = (a[0] * b[1] - a[1] * b[0]) * f;
  out[0] = b[0] * a[2] + a[0] * b[2] - a[1] * k;
  out[1] = b[1] * a[2] + a[1] * b[2] + a[0] * k;
  out[2] = b[2] * a[2] - (a[0] * b[0] + a[1] * b[1]);
}

/* ---------------- spectrum / quantile tables ------------------------------- */

float ppo_spectrum_sample(const float* k, int32_t n, float u) {
  if (n <= 1) return k[0];
  float x = u * (float)n - 0.5f;
  if (x < 0.0f) x = 0.0f;
  if (x > (float)(n - 1)) x = (float)(n - 1);
  int i = (int)floorf(x);
  if (i > n - 2) i = n - 2;
  float f = x - (float)i;
  return k[i] + f * (k[i + 1] - k[i]);
}

float ppo_quantile_sample(const float* q, int32_t n, float u) {
  if (n <= 1) return q[0];
  float x = u * (float)(n - 1);
  int i = (int)floorf(x);
  if (i > n - 2) i = n - 2;
  if (i < 0) i = 0;
  float f = x - (float)i;
  return q[i] + f * (q[i + 1] - q[i]);
}

/* ---------------- gamma (Marsaglia & Tsang 2000) --------------------------- */

float ppo_gamma_f32(int64_t seed, int32_t src, int64_t photon, float shape, float scale,
                    uint32_t* calls_used) {
  float a = shape;
  int boost = 0;
  if (a < 1.0f) { a += 1.0f; boost = 1; }
  float d = a - 1.0f / 3.0f;
  float c = 1.0f / sqrtf(9.0f * d);
  float u[4];
  for (uint32_t j = 0; j < PPO_GAMMA_MAX_TRIES; ++j) {
    ppo_uniforms(seed, src, photon, PPO_EXTRA_CALL + j, u);
    float x = sqrtf(-2.0f * logf(u[0])) * cosf(6.2831855f * u[1]);
    float v = 1.0f + c * x;
    if (v <= 0.0f) continue;
    v = v * v * v;
    float x2 = x * x;
    if (u[2] < 1.0f - 0.0331f * x2 * x2 || logf(u[2]) < 0.5f * x2 + d * (1.0f - v + logf(v))) {
      float gsample = d * v;
      if (boost) gsample *= powf(u[3], 1.0f / shape);
      if (calls_used) *calls_used = j + 1;
      return gsample * scale;
    }
  }
  if (calls_used) *calls_used = PPO_GAMMA_MAX_TRIES;
  return d * scale;
}

static double gamma_f64(int64_t seed, int32_t src, int64_t photon, double shape, double scale) {
  double a = shape;
  int boost = 0;
  if (a < 1.0) { a += 1.0; boost = 1; }
  double d = a - 1.0 / 3.0;
  double c = 1.0 / sqrt(9.0 * d);
  float u[4];
  for (uint32_t j = 0; j < PPO_GAMMA_MAX_TRIES; ++j) {
    ppo_uniforms(seed, src, photon, PPO_EXTRA_CALL + j, u);
    double x = sqrt(-2.0 * log((double)u[0])) * cos(6.283185307179586 * (double)u[1]);
    double v = 1.0 + c * x;
    if (v <= 0.0) continue;
    v = v * v * v;
    double x2 = x * x;
    double uu = (double)u[2];
    if (uu < 1.0 - 0.0331 * x2 * x2 || log(uu) < 0.5 * x2 + d * (1.0 - v + log(v))) {
      double gsample = d * v;
      if (boost) gsample *= pow((double)u[3], 1.0 / shape);
      return gsample * scale;
    }
  }
  return d * scale;
}

/* ---------------- ray-sphere (src/photon_prop_cuda.jl:309-351) ------------- */

int ppo_intersect_sphere_f32(const float c[3], float rsq, const float pos[3], const float dir[3],
                             float step, float* d) {
  float dp0 = pos[0] - c[0], dp1 = pos[1] - c[1], dp2 = pos[2] - c[2];
  float a = dir[0] * dp0 + dir[1] * dp1 + dir[2] * dp2;
  float pp = dp0 * dp0 + dp1 * dp1 + dp2 * dp2;
  float b = a * a - (pp - rsq);
  int isec = b >= 0.0f;
  float dd = isec ? -a - sqrtf(fabsf(b)) : -1.0f;
  if (dd > 0.0f && dd < step) {
    *d = dd;
    return 1;
  }
  return 0;
}

/* The FP32 and FP64 bodies share one source. */
#define REAL float
#define FN(name) name##_f32
#define RSQRT sqrtf
#define RLOG logf
#define RACOS acosf
#define RSIN sinf
#define RCOS cosf
#define RABS fabsf
#define R(x) x##f
#include "pp_oracle_body.inc"
#undef REAL
#undef FN
#undef RSQRT
#undef RLOG
#undef RACOS
#undef RSIN
#undef RCOS
#undef RABS
#undef R

#define REAL double
#define FN(name) name##_f64
#define RSQRT sqrt
#define RLOG log
#define RACOS acos
#define RSIN sin
#define RCOS cos
#define RABS fabs
#define R(x) x
#define PPO_BODY_F64 1
#include "pp_oracle_body.inc"

int32_t ppo_max_threads(void) {
#ifdef _OPENMP
  return (int32_t)omp_get_max_threads();
#else
  return 1;
#endif
}

#include <stddef.h>
#include <string.h>

int64_t ppo_abi_layout(const char* what) {
#define PPO_SIZE(T) if (!strcmp(what, #T)) return (int64_t)sizeof(T);
#define PPO_OFF(T, f) if (!strcmp(what, #T "." #f)) return (int64_t)offsetof(T, f);
  PPO_SIZE(pp_source) PPO_SIZE(pp_sphere) PPO_SIZE(pp_medium) PPO_SIZE(pp_tuning)
  PPO_SIZE(pp_hit_record) PPO_SIZE(pp_counters) PPO_SIZE(pp_target) PPO_SIZE(pp_pmt_target)
  PPO_SIZE(pp_pom_model) PPO_SIZE(pp_dom_model) PPO_SIZE(pp_multipmt_model)
  PPO_SIZE(pp_detection_models) PPO_SIZE(pp_hits)
  PPO_OFF(pp_source, smear_table) PPO_OFF(pp_source, first_photon)
  PPO_OFF(pp_medium, phase_kind) PPO_OFF(pp_medium, hg_g)
  PPO_OFF(pp_hit_record, time) PPO_OFF(pp_hit_record, module_index)
  PPO_OFF(pp_dom_model, polymax) PPO_OFF(pp_dom_model, apply_wl_acceptance) PPO_OFF(pp_dom_model, wl)
  PPO_OFF(pp_multipmt_model, pmt_dir) PPO_OFF(pp_multipmt_model, qe)
  PPO_OFF(pp_pom_model, pmt_dir) PPO_OFF(pp_pom_model, pmt_group)
  PPO_OFF(pp_detection_models, multipmt)
#undef PPO_SIZE
#undef PPO_OFF
  return -1;
}
