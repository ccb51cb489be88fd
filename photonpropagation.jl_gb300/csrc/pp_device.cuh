// pp_device.cuh -- device-side step functions of the photon-transport kernel.
//
// Each function states the PhotonPropagation.jl v0.9.3 function it stands in
// for (paths inside that project).  Every function comes in two precisions of
// the transcendental functions: kPrecise = true uses the IEEE-accurate CUDA
// math library (used by the replay tests), kPrecise = false uses the SFU
// approximations (lg2/ex2/sin/cos/rcp/sqrt .approx), whose absolute error is
// below 1e-6 on the argument ranges used here.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "pp_internal.h"

namespace ppdev {

constexpr uint32_t kPhiloxM0 = 0xD2511F53u;
constexpr uint32_t kPhiloxM1 = 0xCD9E8D57u;
constexpr uint32_t kPhiloxW0 = 0x9E3779B9u;
constexpr uint32_t kPhiloxW1 = 0xBB67AE85u;
constexpr uint32_t kExtraCall = 0x80000000u;  // first call of the emitter stream
constexpr int kGammaMaxTries = 64;
constexpr float kTwoPi = 6.2831855f;           // Float32(2*pi)
constexpr float kPi = 3.14159274f;
constexpr float kCVac = 0.299792458f;          // m/ns

// ---- Philox4x32-10 (Salmon et al., SC'11) --------------------------------
// Counter = (photon lo, photon hi, call, source), key = seed (lo, hi).
__device__ __forceinline__ uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += kPhiloxW0;
      k1 += kPhiloxW1;
    }
    const unsigned long long p0 = (unsigned long long)kPhiloxM0 * c.x;
    const unsigned long long p1 = (unsigned long long)kPhiloxM1 * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1,
                   (uint32_t)p0);
  }
  return c;
}

// The same with the ten rounds' keys given (key + r * (W0, W1), r = 0..9).
__device__ __forceinline__ uint4 philox(uint4 c, const uint32_t* __restrict__ rk) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned long long p0 = (unsigned long long)kPhiloxM0 * c.x;
    const unsigned long long p1 = (unsigned long long)kPhiloxM1 * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ rk[2 * r], (uint32_t)p1,
                   (uint32_t)(p0 >> 32) ^ c.w ^ rk[2 * r + 1], (uint32_t)p0);
  }
  return c;
}

// 24-bit uniform in (0, 1] (exact: integer <= 2^24 times 2^-24).
__device__ __forceinline__ float u01(uint32_t x) {
  return __uint2float_rn((x >> 8) + 1u) * 5.9604644775390625e-8f;
}

// ---- precision-selected primitives -----------------------------------------
__device__ __forceinline__ float approx_sqrt(float x) {
  float y;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float approx_rcp(float x) {
  float y;
  asm("rcp.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float approx_lg2(float x) {
  float y;
  asm("lg2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float approx_ex2(float x) {
  float y;
  asm("ex2.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <bool P>
__device__ __forceinline__ float f_log(float x) {
  if (P) return logf(x);
  return approx_lg2(x) * 0.693147182f;  // ln(x) = log2(x) * ln(2)
}
template <bool P>
__device__ __forceinline__ float f_sqrt(float x) {
  return P ? __fsqrt_rn(x) : approx_sqrt(x);
}
template <bool P>
__device__ __forceinline__ float f_rcp(float x) {
  return P ? __frcp_rn(x) : approx_rcp(x);
}
template <bool P>
__device__ __forceinline__ float f_div(float a, float b) {
  return P ? __fdiv_rn(a, b) : a * approx_rcp(b);
}
// Cube root of a positive number: 2^(log2(x)/3).
template <bool P>
__device__ __forceinline__ float f_cbrt_pos(float x) {
  return P ? cbrtf(x) : approx_ex2(approx_lg2(x) * 0.333333343f);
}
template <bool P>
__device__ __forceinline__ float f_exp(float x) {
  return P ? expf(x) : approx_ex2(x * 1.44269502f);
}
// sin / cos of 2*pi*u for u in (0, 1].  The fast form evaluates the SFU at
// 2*pi*u - pi, inside [-pi, pi] where its error is smallest, and flips signs.
template <bool P>
__device__ __forceinline__ void f_sincos_2pi(float u, float* s, float* c) {
  if (P) {
    sincosf(kTwoPi * u, s, c);
  } else {
    float ss, cc;
    __sincosf(fmaf(kTwoPi, u, -kPi), &ss, &cc);
    *s = -ss;
    *c = -cc;
  }
}
template <bool P>
__device__ __forceinline__ void f_sincos(float x, float* s, float* c) {
  if (P) sincosf(x, s, c); else __sincosf(x, s, c);
}

// a*b + c: fused in the fast variant, two roundings in the replay variant
// (which is compiled without contraction, like the oracle).
template <bool P>
__device__ __forceinline__ float madd(float a, float b, float c) {
  return P ? a * b + c : fmaf(a, b, c);
}

// uniform(minval, maxval) of src/photon_prop_cuda.jl:48-51 on a given uniform.
__device__ __forceinline__ float uniform_ab(float a, float b, float u) { return a + u * (b - a); }

// ---- geometry ----------------------------------------------------------------
// Rotation taking e_z onto the unit vector a, applied to b (rot_from_ez_fast,
// PhysicsTools; called at src/photon_prop_cuda.jl:92-95, :296).  Written in
// the Rodrigues form whose only division is well conditioned in each
// hemisphere of a; the expression order matches the oracle's.
template <bool P>
__device__ __forceinline__ float3 rot_from_ez(float3 a, float3 b) {
  const float s2 = P ? a.x * a.x + a.y * a.y : fmaf(a.y, a.y, a.x * a.x);
  if (s2 == 0.0f) {
    const float sg = a.z >= 0.0f ? 1.0f : -1.0f;
    return make_float3(sg * b.x, sg * b.y, sg * b.z);
  }
  // 1 / (1 + a.z), written as (1 - a.z) / s2 in the lower hemisphere where
  // 1 + a.z cancels; the fast form selects the operands of one reciprocal
  float f;
  if (P) {
    f = a.z >= 0.0f ? f_rcp<P>(1.0f + a.z) : f_div<P>(1.0f - a.z, s2);
  } else {
    const bool up = a.z >= 0.0f;
    f = (up ? 1.0f : 1.0f - a.z) * approx_rcp(up ? 1.0f + a.z : s2);
  }
  if (P) {
    const float k = (a.x * b.y - a.y * b.x) * f;
    return make_float3(b.x * a.z + a.x * b.z - a.y * k, b.y * a.z + a.y * b.z + a.x * k,
                       b.z * a.z - (a.x * b.x + a.y * b.y));
  }
  // the same with every fused multiply-add written out (the fast variant is
  // compiled without automatic contraction, so its rounding is fixed here)
  const float k = fmaf(a.x, b.y, -(a.y * b.x)) * f;
  return make_float3(fmaf(a.x, b.z, fmaf(b.x, a.z, -(a.y * k))),
                     fmaf(a.y, b.z, fmaf(b.y, a.z, a.x * k)),
                     fmaf(b.z, a.z, -fmaf(a.x, b.x, a.y * b.y)));
}

// sph_to_cart(theta, phi) with phi = 2*pi*u_phi.
template <bool P>
__device__ __forceinline__ float3 sph_to_cart(float theta, float u_phi) {
  if (P) {
    const float phi = uniform_ab(0.0f, kTwoPi, u_phi);
    const float st = sinf(theta), ct = cosf(theta);
    return make_float3(st * cosf(phi), st * sinf(phi), ct);
  }
  float st, ct, sp, cp;
  __sincosf(theta, &st, &ct);
  f_sincos_2pi<false>(u_phi, &sp, &cp);
  return make_float3(st * cp, st * sp, ct);
}

// Direction with polar cosine ct and azimuth 2*pi*u_phi.  The replay variant
// goes through theta = acos(ct) as the reference does
// (initialize_direction_isotropic, src/photon_prop_cuda.jl:73-77); the fast
// one uses sin(theta) = sqrt(1 - ct^2).
template <bool P>
__device__ __forceinline__ float3 dir_from_cos(float ct, float u_phi) {
  if (P) return sph_to_cart<true>(acosf(ct), u_phi);
  const float st = approx_sqrt(fmaxf(1.0f - ct * ct, 0.0f));
  float sp, cp;
  f_sincos_2pi<false>(u_phi, &sp, &cp);
  return make_float3(st * cp, st * sp, ct);
}

// ---- tables ------------------------------------------------------------------
// Inverse-CDF spectrum sampled like a 1-D linear-filtered texture with
// normalised coordinates and clamp addressing (src/spectrum.jl:79-83,
// :137-138): texel i sits at (i + 0.5) / n.  FP32 weights instead of the
// texture unit's 8-bit fraction.
__device__ __forceinline__ float spectrum_sample(const float* __restrict__ k, int n, float u) {
  if (n <= 1) return __ldg(k);
  const float x = fminf(fmaxf(u * (float)n - 0.5f, 0.0f), (float)(n - 1));
  const int i = min((int)x, n - 2);
  const float f = x - (float)i;
  const float a = __ldg(k + i), b = __ldg(k + i + 1);
  return a + f * (b - a);
}

// Quantile table with knots at u = i / (n - 1).
__device__ __forceinline__ float quantile_sample(const float* __restrict__ q, int n, float u) {
  if (n <= 1) return __ldg(q);
  const float x = u * (float)(n - 1);
  const int i = min(max((int)x, 0), n - 2);
  const float f = x - (float)i;
  const float a = __ldg(q + i), b = __ldg(q + i + 1);
  return a + f * (b - a);
}

// Medium at wavelength wl: {sca_len, group velocity, abs_len, n}, linear in wl.
__device__ __forceinline__ float4 medium_at(const float4* __restrict__ t, int n, float wl_min,
                                            float inv_step, float wl) {
  const float x = fminf(fmaxf((wl - wl_min) * inv_step, 0.0f), (float)(n - 1));
  const int i = min((int)x, n - 2);
  const float f = x - (float)i;
  const float4 a = __ldg(t + i), b = __ldg(t + i + 1);
  return make_float4(a.x + f * (b.x - a.x), a.y + f * (b.y - a.y), a.z + f * (b.z - a.z),
                     a.w + f * (b.w - a.w));
}

// ---- scattering (update_direction, src/photon_prop_cuda.jl:280-298) ---------
// With probability hg_weight Henyey-Greenstein at g, else the second
// component: Einstein-Smoluchowski at b (MixedHGES, Cardano root of the cubic
// CDF) or simplified Liu at g (cos = 2 eta^((1-g)/(1+g)) - 1, the deep-ice
// mixture).  Both samples are computed and one is selected (a warp almost
// always needs both anyway); the second component's kind is uniform per
// launch.  The fast variant reads the Einstein-Smoluchowski root from the
// medium's table (PhaseDev::es_table) when it has one; the replay variant
// always evaluates the formula.
template <bool P>
__device__ __forceinline__ float scatter_cos(const pp::PhaseDev& ph, float u_choice, float eta) {
  float hg, other;
  if (P) {  // the oracle's expression forms, IEEE division/sqrt/cbrt/pow
    const float g = ph.hg_g, b = ph.es_b;
    const float t = (1.0f - g * g) / (1.0f + g * (2.0f * eta - 1.0f));
    hg = 1.0f / (2.0f * g) * (1.0f + g * g - t * t);
    hg = hg < -1.0f ? -1.0f : (hg > 1.0f ? 1.0f : hg);
    if (ph.kind == PP_PHASE_HG_SL) {
      other = 2.0f * powf(eta, ph.sl_exp) - 1.0f;
    } else {
      const float q = (b + 3.0f) * (eta - 0.5f) / b;
      const float d = sqrtf(q * q + 1.0f / (b * b * b));
      other = cbrtf(q + d) + cbrtf(q - d);
    }
  } else {
    const float t = ph.hg_1mg2 * approx_rcp(fmaf(ph.hg_g, fmaf(2.0f, eta, -1.0f), 1.0f));
    hg = fminf(fmaxf(fmaf(-t, t, ph.hg_1pg2) * ph.hg_inv2g, -1.0f), 1.0f);
    if (ph.kind == PP_PHASE_HG_SL) {
      other = fmaf(2.0f, approx_ex2(ph.sl_exp * approx_lg2(eta)), -1.0f);
    } else if (ph.es_table) {
      // the tabulated inverse CDF, linearly interpolated (eta in (0, 1])
      const float x = eta * (float)pp::kEsTable;
      const int i = min((int)x, pp::kEsTable - 1);
      const float2 t = __ldg(ph.es_table + i);
      other = fmaf(x - (float)i, t.y, t.x);
    } else {
      const float q = ph.es_k1 * (eta - 0.5f);
      const float d = approx_sqrt(fmaf(q, q, ph.es_k2));
      other = f_cbrt_pos<false>(q + d) - f_cbrt_pos<false>(d - q);
    }
  }
  return u_choice < ph.hg_weight ? hg : other;
}

// Back onto the unit sphere, for the fast variant: its SFU sine, cosine and
// square root leave |dir| off 1 by ~1e-6, and the reference's sphere test
// (b = a^2 - (|p - c|^2 - r^2), which assumes |dir| = 1) turns a norm error e
// into a shift 2 e a^2 of b -- at 100 m from a module comparable to r^2, and
// biased: photons then miss distant modules they should hit.  One Newton
// step of 1/sqrt(n2) from 1 (error ~ (n2 - 1)^2) on the FMA pipe.
__device__ __forceinline__ float3 renormalise(float3 d) {
  const float n2 = fmaf(d.z, d.z, fmaf(d.y, d.y, d.x * d.x));
  const float s = fmaf(-0.5f, n2, 1.5f);
  return make_float3(d.x * s, d.y * s, d.z * s);
}

template <bool P>
__device__ __forceinline__ float3 update_direction(const pp::PhaseDev& ph, float3 dir, float u1,
                                                   float u2, float u3) {
  const float c = scatter_cos<P>(ph, u1, u2);
  const float s2 = P ? 1.0f - c * c : fmaf(-c, c, 1.0f);
  const float st = f_sqrt<P>(s2 > 0.0f ? s2 : 0.0f);
  float sp, cp;
  if (P) {
    const float phi = uniform_ab(0.0f, kTwoPi, u3);
    sp = sinf(phi);
    cp = cosf(phi);
  } else {
    f_sincos_2pi<false>(u3, &sp, &cp);
  }
  const float3 out = rot_from_ez<P>(dir, make_float3(cp * st, sp * st, c));
  return P ? out : renormalise(out);
}

// ---- ray-sphere test (_intersect_nsphere, src/photon_prop_cuda.jl:309-343) --
// Hit iff the near intersection lies strictly inside (0, step).  Both
// variants evaluate it exactly as the reference's FP32 expression rounds --
// no fused multiply-adds, IEEE square root: b = a^2 - (|p - c|^2 - r^2)
// cancels heavily for distant spheres, so a different rounding order would
// shift which grazing photons hit (and is not the same everywhere the
// compiler inlines this); the test runs only in the grid walk, so exactness
// costs nothing measurable.
template <bool P>
__device__ __forceinline__ bool sphere_hit(float4 s, float3 pos, float3 dir, float step,
                                           float* d_out) {
  const float dx = __fsub_rn(pos.x, s.x), dy = __fsub_rn(pos.y, s.y), dz = __fsub_rn(pos.z, s.z);
  const float a = __fadd_rn(__fadd_rn(__fmul_rn(dir.x, dx), __fmul_rn(dir.y, dy)),
                            __fmul_rn(dir.z, dz));
  const float pp =
      __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  const float b = __fsub_rn(__fmul_rn(a, a), __fsub_rn(pp, s.w));
  if (b >= 0.0f) {
    const float d = __fsub_rn(-a, __fsqrt_rn(b));
    if (d > 0.0f && d < step) {
      *d_out = d;
      return true;
    }
  }
  return false;
}

// Intersection with target j of a shaped-target list (check_intersection,
// src/photon_prop_cuda.jl:345-404): spheres by the sphere formula above;
// rectangles and discs lie in the plane z = z_j, met at d = (z_j - z) / dir_z
// when 0 <= d <= step and the point is strictly inside the shape.
template <bool P>
__device__ __forceinline__ bool shape_hit(const float4* __restrict__ shapes, int j, float3 pos,
                                          float3 dir, float step, float* d_out) {
  const float4 g = __ldg(shapes + 2 * j);
  const float4 h = __ldg(shapes + 2 * j + 1);
  const int kind = __float_as_int(h.y);
  if (kind == PP_TARGET_SPHERE) return sphere_hit<P>(g, pos, dir, step, d_out);
  if (dir.z == 0.0f) return false;
  const float d = f_div<P>(g.z - pos.z, dir.z);
  if (d < 0.0f || d > step) return false;
  const float x = madd<P>(dir.x, d, pos.x) - g.x;
  const float y = madd<P>(dir.y, d, pos.y) - g.y;
  const bool in = kind == PP_TARGET_RECTANGLE ? (fabsf(x) < g.w && fabsf(y) < h.x)
                                              : (x * x + y * y < g.w);
  if (in) *d_out = d;
  return in;
}

// First target in index order intersected within (0, step): the candidates
// come from a 3-D DDA walk over the uniform grid cells the segment crosses
// between t_lo and t_hi (0 <= t_lo, t_hi <= step: the part of the segment
// that may come near a target; the sphere test itself always uses the whole
// segment) (Amanatides & Woo); among all intersected candidates the smallest index
// wins, which is exactly the reference's "first target in index order"
// (src/photon_prop_cuda.jl:497-506).  Returns the 0-based index or -1.
template <bool P>
__device__ __forceinline__ int first_hit(const pp::GridDev& g, const uint32_t* __restrict__ cells,
                                         const uint16_t* __restrict__ items,
                                         const float4* __restrict__ sph, float3 pos, float3 dir,
                                         float step, float t_lo, float t_hi, float* d_out) {
  // Reciprocal direction; zero components become a huge value of the same
  // sign as the step direction chosen below (+ for +0 and -0 alike).
  const float ix = approx_rcp(fabsf(dir.x) > 1e-20f ? dir.x : 1e-20f);
  const float iy = approx_rcp(fabsf(dir.y) > 1e-20f ? dir.y : 1e-20f);
  const float iz = approx_rcp(fabsf(dir.z) > 1e-20f ? dir.z : 1e-20f);
  // Clip the segment to the grid box (slab test).
  const float tx0 = (g.lo[0] - pos.x) * ix, tx1 = (g.hi[0] - pos.x) * ix;
  const float ty0 = (g.lo[1] - pos.y) * iy, ty1 = (g.hi[1] - pos.y) * iy;
  const float tz0 = (g.lo[2] - pos.z) * iz, tz1 = (g.hi[2] - pos.z) * iz;
  const float tmin = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), t_lo));
  const float tmax = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), t_hi));
  if (!(tmin <= tmax)) return -1;

  const int nx = g.dims[0], ny = g.dims[1], nz = g.dims[2];
  int cx = (int)floorf((fmaf(dir.x, tmin, pos.x) - g.lo[0]) * g.inv_cell[0]);
  int cy = (int)floorf((fmaf(dir.y, tmin, pos.y) - g.lo[1]) * g.inv_cell[1]);
  int cz = (int)floorf((fmaf(dir.z, tmin, pos.z) - g.lo[2]) * g.inv_cell[2]);
  cx = min(max(cx, 0), nx - 1);
  cy = min(max(cy, 0), ny - 1);
  cz = min(max(cz, 0), nz - 1);
  const int sx = ix >= 0.0f ? 1 : -1;
  const int sy = iy >= 0.0f ? 1 : -1;
  const int sz = iz >= 0.0f ? 1 : -1;
  float tnx = (fmaf((float)(cx + (sx > 0)), g.cell[0], g.lo[0]) - pos.x) * ix;
  float tny = (fmaf((float)(cy + (sy > 0)), g.cell[1], g.lo[1]) - pos.y) * iy;
  float tnz = (fmaf((float)(cz + (sz > 0)), g.cell[2], g.lo[2]) - pos.z) * iz;
  const float tdx = g.cell[0] * fabsf(ix);
  const float tdy = g.cell[1] * fabsf(iy);
  const float tdz = g.cell[2] * fabsf(iz);
  const int strx = sx, stry = sy * nx, strz = sz * nx * ny;
  int cidx = (cz * ny + cy) * nx + cx;

  int best = 0x7fffffff;
  float best_d = 0.0f;
  const int max_iter = nx + ny + nz + 3;
  for (int it = 0; it < max_iter; ++it) {
    const uint32_t w = cells[cidx];
    const uint32_t cnt = w >> pp::kCellStartBits;
    if (cnt) {
      const uint32_t first = w & pp::kCellStartMask;
      for (uint32_t k = 0; k < cnt; ++k) {
        const int j = items[first + k];
        float d;
        if (j < best && sphere_hit<P>(sph[j], pos, dir, step, &d)) {
          best = j;
          best_d = d;
        }
      }
    }
    // the axis whose boundary comes first (x, then y, on ties), stepped by
    // selects: lanes of a warp step different axes without diverging
    const bool ax = tnx <= tny && tnx <= tnz;
    const bool ay = !ax && tny <= tnz;
    const bool az = !ax && !ay;
    const float tn = ax ? tnx : (ay ? tny : tnz);
    if (tn > tmax) break;
    cx += ax ? sx : 0;
    cy += ay ? sy : 0;
    cz += az ? sz : 0;
    if ((unsigned)cx >= (unsigned)nx || (unsigned)cy >= (unsigned)ny ||
        (unsigned)cz >= (unsigned)nz)
      break;
    tnx += ax ? tdx : 0.0f;
    tny += ay ? tdy : 0.0f;
    tnz += az ? tdz : 0.0f;
    cidx += ax ? strx : (ay ? stry : strz);
  }
  if (best == 0x7fffffff) return -1;
  *d_out = best_d;
  return best;
}

// ---- emitters (initialize_photon_state, src/photon_prop_cuda.jl:158-276) ----

// Gamma(shape, scale) by Marsaglia & Tsang (2000) from the photon's emitter
// stream (rand_gamma, PhysicsTools; called at :214).
template <bool P>
__device__ __forceinline__ float gamma_sample(float shape, float scale, uint32_t plo, uint32_t phi,
                                              uint32_t src, uint32_t k0, uint32_t k1) {
  float a = shape;
  const bool boost = a < 1.0f;
  if (boost) a += 1.0f;
  const float d = a - 1.0f / 3.0f;
  const float c = P ? 1.0f / sqrtf(9.0f * d) : rsqrtf(9.0f * d);
  for (int j = 0; j < kGammaMaxTries; ++j) {
    const uint4 r = philox(make_uint4(plo, phi, kExtraCall + (uint32_t)j, src), k0, k1);
    const float u0 = u01(r.x), u1 = u01(r.y), u2 = u01(r.z);
    float cs;
    if (P) {
      cs = cosf(kTwoPi * u1);
    } else {
      float sn;
      f_sincos_2pi<false>(u1, &sn, &cs);
    }
    const float x = f_sqrt<P>(-2.0f * f_log<P>(u0)) * cs;
    float v = 1.0f + c * x;
    if (v <= 0.0f) continue;
    v = v * v * v;
    const float x2 = x * x;
    if (u2 < 1.0f - 0.0331f * x2 * x2 || f_log<P>(u2) < 0.5f * x2 + d * (1.0f - v + f_log<P>(v))) {
      float gs = d * v;
      if (boost) gs *= (P ? powf(u01(r.w), 1.0f / shape) : f_exp<false>(f_log<false>(u01(r.w)) / shape));
      return gs * scale;
    }
  }
  return d * scale;
}

// Cherenkov cone about the emitter axis: theta_c = acos(1/n), phi ~ U(0, 2pi),
// optionally rotated onto a sampled track direction first
// (sample_cherenkov_direction, :80-111).
template <bool P>
__device__ __forceinline__ float3 cherenkov_dir(float3 axis, float ref_ix, float u_phi,
                                                float u_track, float u_track_phi, bool smear,
                                                const float* __restrict__ track, int n_track) {
  float3 ph = P ? sph_to_cart<true>(acosf(1.0f / ref_ix), u_phi)
                : dir_from_cos<false>(approx_rcp(ref_ix), u_phi);
  if (smear) {
    float ct = quantile_sample(track, n_track, u_track);
    ct = ct > 1.0f ? 1.0f : (ct < -1.0f ? -1.0f : ct);
    ph = rot_from_ez<P>(dir_from_cos<P>(ct, u_track_phi), ph);
  }
  return rot_from_ez<P>(axis, ph);
}

}  // namespace ppdev
