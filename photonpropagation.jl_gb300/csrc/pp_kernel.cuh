// pp_kernel.cuh -- the persistent photon-propagation kernel template.
//
// Included by two translation units: pp_propagate.cu instantiates the fast
// variant (SFU approximations, FMA contraction), pp_propagate_precise.cu the
// replay variant (IEEE math library, compiled with -fmad=false so that every
// FP32 expression rounds exactly as the CPU oracle's does).
//
// Replaces cuda_propagate_photons! (PhotonPropagation.jl v0.9.3,
// src/photon_prop_cuda.jl:429-549) and its one-launch-per-source host loop
// (:927-943).  Design:
//   * persistent CTAs; every warp pulls chunks of 32 * photons_per_thread
//     photons of one source from a device work queue, so one launch covers any
//     number of sources with uneven photon counts;
//   * photon i of source s draws its random numbers from Philox4x32-10 at
//     counter (i, call, s) and key = seed: results do not depend on the launch
//     shape and any photon range can be replayed;
//   * speculative stepping with deferred hit tests.  Each lane runs all
//     n_steps of its photon without waiting for the target test.  A step
//     segment is cleared cheaply when the safety field proves that no target
//     lies within the ball around its midpoint; the rare uncleared segments
//     go to a per-warp queue in shared memory.  When 32 of them wait, the warp
//     clips them, one per lane, by sphere tracing the safety field from both
//     ends (most vanish); the survivors stay queued with the part of the
//     segment that may come near a target, and whenever 32 survivors wait the
//     warp walks them, one per lane, through the uniform-grid DDA over that
//     part only.  The photon's hit is the earliest step with an intersection
//     and, within it, the lowest target index -- the reference's "first
//     target in index order" (:497-506).  Steps after the hit were computed
//     speculatively and are discarded;
//   * the target grid (cells, candidate lists, spheres) is staged once per CTA
//     into shared memory with a TMA bulk copy completing on an mbarrier, waited
//     on with a time bound;
//   * hits are appended with one atomic per warp into 80-byte records written
//     as five 16-byte vector stores.
#pragma once

#include <cuda_runtime.h>

#include "pp_device.cuh"
#include "pp_internal.h"

namespace pp {
namespace {

using namespace ppdev;

__device__ __forceinline__ unsigned long long global_timer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long* u64(uint64_t* p) {
  return reinterpret_cast<unsigned long long*>(p);
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Issue TMA bulk copies of `bytes` (multiple of 16, both ends 16-byte
// aligned) completing on the mbarrier at bar_a.
__device__ __forceinline__ void bulk_copy(unsigned char* dst, const unsigned char* src,
                                          uint32_t bytes, uint32_t bar_a) {
  constexpr uint32_t kChunk = 32768;
  for (uint32_t off = 0; off < bytes; off += kChunk) {
    const uint32_t n = bytes - off < kChunk ? bytes - off : kChunk;
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst + off)),
        "l"(src + off), "r"(n), "r"(bar_a)
        : "memory");
  }
}

// Stage two global tables into shared memory with TMA bulk copies completing
// on one mbarrier.  Every thread then waits on the barrier's phase 0 for at
// most limit_ns.  Returns false on timeout.  skip_copies (a diagnostic, see
// pp_debug_staging_timeout) arms the barrier but issues no copy, so that the
// bounded wait runs out with nothing in flight.
__device__ bool stage_tables(unsigned char* dst0, const unsigned char* src0, uint32_t bytes0,
                             unsigned char* dst1, const unsigned char* src1, uint32_t bytes1,
                             unsigned long long* bar, unsigned long long limit_ns,
                             bool skip_copies) {
  const uint32_t bar_a = smem_addr(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar_a), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_a),
                 "r"(bytes0 + bytes1)
                 : "memory");
    if (!skip_copies) {
      bulk_copy(dst0, src0, bytes0, bar_a);
      bulk_copy(dst1, src1, bytes1, bar_a);
    }
  }
  const unsigned long long t0 = global_timer_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar_a), "r"(0)
        : "memory");
    if (done) return true;
    if (global_timer_ns() - t0 > limit_ns) return false;
  }
}

// Field cell nearest to m (clamped to the field): its index, and m's offset
// from the cell's centre.
__device__ __forceinline__ int field_cell(const SafetyDev& s, float3 m, float3* off) {
  const float fx = fminf(fmaxf(floorf(fmaf(m.x, s.inv_cell, -s.lo_sc[0])), 0.0f), s.fmaxc[0]);
  const float fy = fminf(fmaxf(floorf(fmaf(m.y, s.inv_cell, -s.lo_sc[1])), 0.0f), s.fmaxc[1]);
  const float fz = fminf(fmaxf(floorf(fmaf(m.z, s.inv_cell, -s.lo_sc[2])), 0.0f), s.fmaxc[2]);
  *off = make_float3(fmaf(fx, s.cell, s.c_lo[0]) - m.x, fmaf(fy, s.cell, s.c_lo[1]) - m.y,
                     fmaf(fz, s.cell, s.c_lo[2]) - m.z);
  return (int)fmaf(fmaf(fz, s.fdims[1], fy), s.fdims[0], fx);
}

// Stored lower bound of a field cell in metres: the byte b becomes a float
// through its bit pattern (2^23 + b), exactly.
template <bool kShared>
__device__ __forceinline__ float field_value(const unsigned char* __restrict__ f, int idx) {
  const uint32_t b = kShared ? f[idx] : __ldg(f + idx);
  return fmaf(__uint_as_float(0x4B000000u | b), kSafetyQuantum, -8388608.0f * kSafetyQuantum);
}

// True when the safety field proves that no (inflated) target sphere meets
// the ball of radius R about m.  Branch-free: two lower bounds on the distance
// from m to every target, of which one must exceed R --
//   the Chebyshev distance from m to the field's box (which contains every
//   target; it is below the Euclidean distance), and
//   D(c) - |m - c| for the centre c of the field cell nearest to m (distance
//   to the targets is 1-Lipschitz; D(c) is stored quantised down).
template <bool kShared>
__device__ __forceinline__ bool ball_clear(const SafetyDev& s, const unsigned char* __restrict__ f,
                                           float3 m, float R) {
  const float box = fmaxf(fmaxf(fabsf(m.x - s.bc[0]) - s.he[0], fabsf(m.y - s.bc[1]) - s.he[1]),
                          fabsf(m.z - s.bc[2]) - s.he[2]);
  float3 o;
  const int idx = field_cell(s, m, &o);
  const float budget = field_value<kShared>(f, idx) - R;
  return box > R || (budget > 0.0f && fmaf(o.z, o.z, fmaf(o.y, o.y, o.x * o.x)) < budget * budget);
}

// The segment pos + t*dir, t in [0, L], provably misses every target: it lies
// inside the ball of radius L/2 about its midpoint.
template <bool kShared>
__device__ __forceinline__ bool segment_clear(const SafetyDev& s, const unsigned char* f,
                                              float3 pos, float3 dir, float L) {
  const float h = 0.5f * L;
  return ball_clear<kShared>(
      s, f, make_float3(fmaf(dir.x, h, pos.x), fmaf(dir.y, h, pos.y), fmaf(dir.z, h, pos.z)),
      fmaf(h, 1.0001f, 1e-4f));
}

// Lower bound on the distance from m to every (inflated) target sphere:
// D(c) - |m - c| for the field cell c nearest to m (distance is 1-Lipschitz,
// D(c) is stored quantised down).  Valid for any m; weak (often negative) far
// outside the field's box.
template <bool kShared, bool P>
__device__ __forceinline__ float field_bound(const SafetyDev& s, const unsigned char* __restrict__ f,
                                             float3 m) {
  float3 o;
  const int idx = field_cell(s, m, &o);
  return field_value<kShared>(f, idx) - f_sqrt<P>(fmaf(o.z, o.z, fmaf(o.y, o.y, o.x * o.x)));
}

// Slack (m) taken off each clipped end: covers the rounding of the traced
// points and of the square root, well inside the 1 cm by which the field's
// spheres are inflated.
constexpr float kClipSlack = 5e-3f;

// Clip the unchecked queue entries [n2, n2 + n1) (n1 <= 32, one per lane):
// first to the grid's box (no target lies outside it), then by sphere tracing
// the safety field twice from each end of what is left -- no target lies
// within field_bound(p) of a point p -- so the walk can skip [0, t0) and
// (t1, L].  Entries left with t0 < t1 are compacted (in place) to
// [n2, n2 + kept) with their interval; the others cannot hit anything and are
// dropped.  Returns the new number of checked entries.
template <bool kShared, bool P>
__device__ __forceinline__ int check_queue(WarpQueue& q, int n2, int n1, const GridDev& g,
                                           const SafetyDev& s, const unsigned char* __restrict__ f,
                                           int lane) {
  const int src = n2 + lane;
  bool keep = false;
  float3 p = make_float3(0.0f, 0.0f, 0.0f), d = p;
  float L = 0.0f, d0 = 0.0f, t0 = 0.0f, t1 = 0.0f;
  uint32_t meta = 0;
  if (lane < n1) {
    p = make_float3(q.px[src], q.py[src], q.pz[src]);
    d = make_float3(q.dx[src], q.dy[src], q.dz[src]);
    L = q.len[src];
    // slab test against the grid box (the same one the walk clips to)
    const float ix = approx_rcp(fabsf(d.x) > 1e-20f ? d.x : 1e-20f);
    const float iy = approx_rcp(fabsf(d.y) > 1e-20f ? d.y : 1e-20f);
    const float iz = approx_rcp(fabsf(d.z) > 1e-20f ? d.z : 1e-20f);
    const float tx0 = (g.lo[0] - p.x) * ix, tx1 = (g.hi[0] - p.x) * ix;
    const float ty0 = (g.lo[1] - p.y) * iy, ty1 = (g.hi[1] - p.y) * iy;
    const float tz0 = (g.lo[2] - p.z) * iz, tz1 = (g.hi[2] - p.z) * iz;
    t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), L));
#pragma unroll
    for (int it = 0; it < 2; ++it) {
      t0 += fmaxf(field_bound<kShared, P>(s, f,
                                          make_float3(fmaf(d.x, t0, p.x), fmaf(d.y, t0, p.y),
                                                      fmaf(d.z, t0, p.z))),
                  0.0f);
      t1 -= fmaxf(field_bound<kShared, P>(s, f,
                                          make_float3(fmaf(d.x, t1, p.x), fmaf(d.y, t1, p.y),
                                                      fmaf(d.z, t1, p.z))),
                  0.0f);
    }
    t0 = fmaxf(t0 - kClipSlack, 0.0f);
    t1 = fminf(t1 + kClipSlack, L);
    keep = t0 < t1;
    d0 = q.dist0[src];
    meta = q.meta[src];
  }
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  __syncwarp();  // every entry is read before any is overwritten
  if (keep) {
    const int dst = n2 + __popc(m & ((1u << lane) - 1u));
    q.px[dst] = p.x;
    q.py[dst] = p.y;
    q.pz[dst] = p.z;
    q.dx[dst] = d.x;
    q.dy[dst] = d.y;
    q.dz[dst] = d.z;
    q.len[dst] = L;
    q.dist0[dst] = d0;
    q.meta[dst] = meta;
    q.t0[dst] = t0;
    q.t1[dst] = t1;
  }
  __syncwarp();
  return n2 + __popc(m);
}

// Test the checked entries [base, base + c) (c <= 32): lane e walks entry
// base + e through the grid DDA over its clipped interval -- or, when at most
// 16 (10) entries are left, two (three) lanes walk an equal slice of each
// entry's interval, overlapping by the clip slack, so that the longest walk
// sets the pass's length less often; the earliest
// (step, target) per owner lane wins via a shared atomicMin on the key
// (step << 16 | target), and the winning lane writes the hit state into the
// owner's slot.
template <bool P>
__device__ __forceinline__ void test_queue(WarpQueue& q, WarpBest& b, int base, int c,
                                           const GridDev& g, const uint32_t* cells,
                                           const uint16_t* items, const float4* sph, int lane) {
  // with few entries, m lanes share one entry, each walking 1/m of its interval
  const int m = c <= 10 ? 3 : (c <= 16 ? 2 : 1);
  const int el = lane / m, piece = lane - el * m;
  const int e = base + el;
  int j = -1, owner = 0;
  uint32_t key = 0;
  float d = 0.0f, d0 = 0.0f;
  float3 p = make_float3(0.0f, 0.0f, 0.0f), dir = p;
  if (el < c) {
    p = make_float3(q.px[e], q.py[e], q.pz[e]);
    dir = make_float3(q.dx[e], q.dy[e], q.dz[e]);
    d0 = q.dist0[e];
    const uint32_t meta = q.meta[e];
    owner = (int)(meta & 31u);
    const float t0 = q.t0[e], t1 = q.t1[e];
    const float w = (t1 - t0) * (m == 1 ? 1.0f : (m == 2 ? 0.5f : 0.33333334f));
    const float ta = piece == 0 ? t0 : fmaxf(fmaf((float)piece, w, t0) - kClipSlack, t0);
    const float tb = piece == m - 1 ? t1 : fminf(fmaf((float)(piece + 1), w, t0) + kClipSlack, t1);
    j = first_hit<P>(g, cells, items, sph, p, dir, q.len[e], ta, tb, &d);
    if (j >= 0) {
      key = ((meta >> 8) << 16) | (uint32_t)j;
      atomicMin(&b.key[owner], key);
    }
  }
  __syncwarp();
  if (j >= 0 && b.key[owner] == key) {
    b.hx[owner] = madd<P>(dir.x, d, p.x);
    b.hy[owner] = madd<P>(dir.y, d, p.y);
    b.hz[owner] = madd<P>(dir.z, d, p.z);
    b.ox[owner] = dir.x;
    b.oy[owner] = dir.y;
    b.oz[owner] = dir.z;
    b.dist[owner] = d0 + d;
  }
  __syncwarp();
}

// Append one hit: one atomic per warp for all lanes that record in this pass;
// the record is written as five 16-byte stores in pp_hit_record's order.
__device__ __forceinline__ void record_hit(const LaunchArgs& a, float3 pos, float wl, float3 dir,
                                           float dist, float3 idir, float abs_w, double time,
                                           long long photon, int module_index, int n_steps,
                                           int source_index, bool* overflowed) {
  const unsigned act = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(act) - 1;
  const unsigned rank = __popc(act & ((1u << lane) - 1u));
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(u64(&a.counters->n_hits), (unsigned long long)__popc(act));
  base = __shfl_sync(act, base, leader);
  const unsigned long long slot = base + rank;
  if (slot < a.capacity) {
    float4* r = reinterpret_cast<float4*>(a.hits + slot);
    r[0] = make_float4(pos.x, pos.y, pos.z, wl);
    r[1] = make_float4(dir.x, dir.y, dir.z, __int_as_float(module_index));
    r[2] = make_float4(dist, idir.x, idir.y, idir.z);
    r[3] = make_float4(abs_w, __int_as_float(n_steps), __int_as_float(source_index), 0.0f);
    reinterpret_cast<double2*>(r)[4] = make_double2(time, __longlong_as_double(photon));
  } else {
    atomicOr(&a.counters->err_flags, (unsigned)PP_FLAG_OVERFLOW);
    *overflowed = true;
  }
}

// Initial state of photon p of source s (initialize_photon_state,
// src/photon_prop_cuda.jl:158-276): position, direction, emission time,
// wavelength and the medium at that wavelength {sca_len, v_group, abs_len,
// n}.  Deterministic in (p, s), so the step loop keeps only what it needs and
// the few photons that hit recompute the rest when their hit is recorded.
struct PhotonInit {
  float3 pos, dir;
  float t0, wl;
  float4 med;
};

template <bool kPrecise>
__device__ __forceinline__ PhotonInit init_photon(const LaunchArgs& a, int s, uint32_t plo,
                                                  uint32_t phi) {
  const pp_source* sp = a.sources + s;
  const int kind = __ldg(&sp->kind);
  const float3 spos = make_float3(__ldg(&sp->position[0]), __ldg(&sp->position[1]),
                                  __ldg(&sp->position[2]));
  const float3 saxis = make_float3(__ldg(&sp->direction[0]), __ldg(&sp->direction[1]),
                                   __ldg(&sp->direction[2]));
  const float stime = __ldg(&sp->time);
  const uint4 r0 = philox(make_uint4(plo, phi, 0u, (uint32_t)s), a.round_keys);
  const float u0 = u01(r0.x), u1 = u01(r0.y), u2 = u01(r0.z), u3 = u01(r0.w);
  const float wl = a.spectrum ? spectrum_sample(a.spectrum, a.n_spectrum, u0)
                              : a.mono_wavelength;
  const float4 med = medium_at(a.medium, a.n_medium, a.med_wl_min, a.med_inv_step, wl);

  // ---- initial state (initialize_photon_state) ----
  float3 pos = spos, dir;
  float t0 = stime;
  switch (kind) {
    case PP_SRC_POINTLIKE_ISOTROPIC:
    case PP_SRC_POINTLIKE_TIME_RANGE:
      dir = dir_from_cos<kPrecise>(uniform_ab(-1.0f, 1.0f, u1), u2);
      if (kind == PP_SRC_POINTLIKE_TIME_RANGE)
        t0 = uniform_ab(stime, __ldg(&sp->time_end), u3);
      break;
    case PP_SRC_COLLIMATED_ISOTROPIC:
      dir = dir_from_cos<kPrecise>(uniform_ab(__ldg(&sp->cut_angle_cos), 1.0f, u2), u1);
      break;
    case PP_SRC_PENCIL: {
      const float div = __ldg(&sp->beam_divergence);
      dir = div > 0.0f ? rot_from_ez<kPrecise>(
                             saxis, sph_to_cart<kPrecise>(
                                        f_sqrt<kPrecise>(uniform_ab(0.0f, div * div, u1)), u2))
                       : saxis;
      break;
    }
    case PP_SRC_AXICONE: {
      float th = __ldg(&sp->angle);
      const float div = __ldg(&sp->beam_divergence);
      if (div > 0.0f) {
        float cs;
        if (kPrecise) {
          cs = cosf(kTwoPi * u3);
        } else {
          float sn;
          f_sincos_2pi<false>(u3, &sn, &cs);
        }
        th += f_sqrt<kPrecise>(-2.0f * f_log<kPrecise>(u2)) * cs * div;
      }
      dir = rot_from_ez<kPrecise>(saxis, sph_to_cart<kPrecise>(th, u1));
      break;
    }
    case PP_SRC_EXTENDED_CHERENKOV:
    case PP_SRC_EXTENDED_CHERENKOV_NOSMEAR:
    case PP_SRC_POINTLIKE_CHERENKOV:
    case PP_SRC_CHERENKOV_TRACK: {
      float along = 0.0f;
      if (kind == PP_SRC_EXTENDED_CHERENKOV || kind == PP_SRC_EXTENDED_CHERENKOV_NOSMEAR) {
        along = gamma_sample<kPrecise>(__ldg(&sp->long_a), 1.0f / __ldg(&sp->long_b), plo, phi,
                                       (uint32_t)s, a.key0, a.key1) *
                __ldg(&sp->long_lrad);
      } else if (kind == PP_SRC_CHERENKOV_TRACK) {
        const uint4 re = philox(make_uint4(plo, phi, kExtraCall, (uint32_t)s), a.round_keys);
        along = uniform_ab(0.0f, __ldg(&sp->length), u01(re.x));
      }
      if (kind != PP_SRC_POINTLIKE_CHERENKOV) {
        pos = make_float3(spos.x + along * saxis.x, spos.y + along * saxis.y,
                          spos.z + along * saxis.z);
        t0 = stime + along / kCVac;
      }
      dir = cherenkov_dir<kPrecise>(
          saxis, med.w, u1, u2, u3, kind != PP_SRC_EXTENDED_CHERENKOV_NOSMEAR,
          a.track + (size_t)__ldg(&sp->smear_table) * (size_t)a.n_track, a.n_track);
      break;
    }
    default:
      dir = make_float3(0.0f, 0.0f, 1.0f);
      break;
  }

  PhotonInit in;
  in.pos = pos;
  in.dir = kPrecise ? dir : renormalise(dir);
  in.t0 = t0;
  in.wl = wl;
  in.med = med;
  return in;
}

// The same as a call, for the hit record (rare): keeps the emission data out
// of the step loop's registers.
template <bool kPrecise>
__device__ __noinline__ PhotonInit init_photon_again(const LaunchArgs& a, int s, uint32_t plo,
                                                     uint32_t phi) {
  return init_photon<kPrecise>(a, s, plo, phi);
}

// One CTA of kMaxBlockThreads per SM caps the kernel at 64 registers.
#ifndef PP_PROPAGATE_MIN_BLOCKS
#define PP_PROPAGATE_MIN_BLOCKS 1
#endif

// kShapes: shaped targets (a.shapes), every target tested at every step in
// index order (no grid, no deferred queue); a list of detector lines is
// searched line by line (src/photon_prop_cuda.jl:611-634).
template <bool kPrecise, bool kSmemGrid, bool kShapes = false>
__global__ void __launch_bounds__(kMaxBlockThreads, PP_PROPAGATE_MIN_BLOCKS)
    propagate_kernel(const __grid_constant__ LaunchArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) unsigned long long bar;

  const uint32_t* cells;
  const uint16_t* items;
  const float4* sph;
  const unsigned char* field;
  if (kSmemGrid) {
    if (!stage_tables(smem, a.blob, a.grid.blob_bytes, smem + a.safety_offset, a.safety,
                      a.sgrid.bytes, &bar, a.wait_limit_ns, a.skip_staging_copies != 0)) {
      atomicOr(&a.counters->err_flags, (unsigned)PP_FLAG_TIMEOUT);
      return;
    }
    cells = reinterpret_cast<const uint32_t*>(smem);
    items = reinterpret_cast<const uint16_t*>(smem + a.grid.off_items);
    sph = reinterpret_cast<const float4*>(smem + a.grid.off_spheres);
    field = smem + a.safety_offset;
  } else {
    cells = reinterpret_cast<const uint32_t*>(a.blob);
    items = reinterpret_cast<const uint16_t*>(a.blob + a.grid.off_items);
    sph = reinterpret_cast<const float4*>(a.blob + a.grid.off_spheres);
    field = a.safety;
  }
  const bool have_grid = a.grid.n_targets > 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpQueue& q = reinterpret_cast<WarpQueue*>(smem + a.state_offset)[warp];
  WarpBest& best = reinterpret_cast<WarpBest*>(smem + a.state_offset +
                                               a.warps_per_block * sizeof(WarpQueue))[warp];
  const unsigned lanemask_lt = (1u << lane) - 1u;

  unsigned long long steps_acc = 0, sim_acc = 0;

  while (true) {
    unsigned long long c = 0;
    unsigned stop = 0;
    if (lane == 0) {
      c = atomicAdd(u64(&a.counters->work_next), 1ull);
      stop = *reinterpret_cast<volatile unsigned*>(&a.counters->err_flags) & PP_FLAG_OVERFLOW;
    }
    c = __shfl_sync(0xffffffffu, c, 0);
    stop = __shfl_sync(0xffffffffu, stop, 0);
    if (c >= a.total_chunks || stop) break;

    // Source owning chunk c: last s with chunk_prefix[s] <= c.
    int lo = 0, hi = a.n_src;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(a.chunk_prefix + mid) <= c) lo = mid; else hi = mid;
    }
    const int s = lo;
    const long long p0 = (long long)(c - __ldg(a.chunk_prefix + s)) * a.chunk_photons;
    const long long pend = min(p0 + (long long)a.chunk_photons, __ldg(a.src_photons + s));
    const long long first = __ldg(&a.sources[s].first_photon);

    for (long long base = p0; base < pend; base += 32) {
      const bool active = base + lane < pend;
      // Lanes past the end replay the first photon of the round (never recorded).
      const long long p = first + (active ? base + lane : base);
      const uint32_t plo = (uint32_t)p, phi = (uint32_t)((unsigned long long)p >> 32);
      float3 pos, dir;
      float sca_len;
      {
        const PhotonInit in = init_photon<kPrecise>(a, s, plo, phi);
        pos = in.pos;
        dir = in.dir;
        sca_len = in.med.x;
      }
      float dist = 0.0f, comp = 0.0f;  // Kahan-compensated path length
      best.key[lane] = 0xffffffffu;
      __syncwarp();
      // warp-uniform queue state: [0, n2) clipped, [n2, n2 + n1) not yet
      int n1 = 0, n2 = 0;
      bool found = false;  // shaped targets: the photon has hit
      // The step loop holds no grid walk: when more than 31 checked entries
      // wait, it stops before appending step k's entries, the walk below takes
      // 32 of them, and the loop resumes at step k (recomputing its random
      // numbers and ball test, which are the same).  At the end of the steps
      // the same walk takes everything left.
      int k = 1;
      while (true) {
      bool flush = true;
      for (; k <= a.n_steps; ++k) {
        const uint4 r = philox(make_uint4(plo, phi, (uint32_t)k, (uint32_t)s), a.round_keys);
        const float step = -f_log<kPrecise>(u01(r.x)) * sca_len;
        if constexpr (kShapes) {
          if (active && !found) {
            int hit = -1;  // 0-based module index to report
            float d = 0.0f;
            int line_no = 0;
            for (int j = 0; j < a.n_shapes; ++j) {
              const float4 h = __ldg(a.shapes + 2 * j + 1);
              if (__float_as_int(h.y) == PP_TARGET_LINE) {
                // DetectorLines: the 2-D test of the line, then its modules;
                // the first crossed line ends the search
                const int nm = __float_as_int(h.x);
                ++line_no;
                float dl;
                if (!sphere_hit<kPrecise>(__ldg(a.shapes + 2 * j), make_float3(pos.x, pos.y, 0.0f),
                                          make_float3(dir.x, dir.y, 0.0f), step, &dl)) {
                  j += nm;
                  continue;
                }
                for (int m = 1; m <= nm; ++m) {
                  if (shape_hit<kPrecise>(a.shapes, j + m, pos, dir, step, &d)) {
                    hit = m + nm * line_no - 1;
                    break;
                  }
                }
                break;
              }
              if (shape_hit<kPrecise>(a.shapes, j, pos, dir, step, &d)) {
                hit = j;
                break;
              }
            }
            if (hit >= 0) {
              found = true;
              best.key[lane] = ((uint32_t)k << 16) | (uint32_t)hit;
              best.hx[lane] = madd<kPrecise>(dir.x, d, pos.x);
              best.hy[lane] = madd<kPrecise>(dir.y, d, pos.y);
              best.hz[lane] = madd<kPrecise>(dir.z, d, pos.z);
              best.ox[lane] = dir.x;
              best.oy[lane] = dir.y;
              best.oz[lane] = dir.z;
              best.dist[lane] = (dist - comp) + d;
            }
          }
        } else {
        const bool need = have_grid && active && !segment_clear<kSmemGrid>(a.sgrid, field, pos, dir, step);
        const unsigned m = __ballot_sync(0xffffffffu, need);
        if (m) {
          const int nn = __popc(m);
          if (n1 + nn > 32) {
            // clip the unchecked entries; walk the grid once 32 checked ones wait
            n2 = check_queue<kSmemGrid, kPrecise>(q, n2, n1, a.grid, a.sgrid, field, lane);
            n1 = 0;
            if (n2 >= 32) {
              flush = false;
              break;
            }
          }
          if (need) {
            const int e = n2 + n1 + __popc(m & lanemask_lt);
            q.px[e] = pos.x;
            q.py[e] = pos.y;
            q.pz[e] = pos.z;
            q.dx[e] = dir.x;
            q.dy[e] = dir.y;
            q.dz[e] = dir.z;
            q.len[e] = step;
            q.dist0[e] = dist - comp;
            q.meta[e] = (uint32_t)lane | ((uint32_t)k << 8);
          }
          n1 += nn;
          __syncwarp();
        }
        }  // kShapes
        pos = make_float3(madd<kPrecise>(dir.x, step, pos.x), madd<kPrecise>(dir.y, step, pos.y),
                          madd<kPrecise>(dir.z, step, pos.z));
        {
          const float y = step - comp, t = dist + y;
          comp = (t - dist) - y;
          dist = t;
        }
        dir = update_direction<kPrecise>(a.phase, dir, u01(r.y), u01(r.z), u01(r.w));
      }
      if (kShapes) break;
      if (flush && n1 > 0) {
        n2 = check_queue<kSmemGrid, kPrecise>(q, n2, n1, a.grid, a.sgrid, field, lane);
        n1 = 0;
      }
      while (n2 > 0) {
        const int c = n2 < 32 ? n2 : 32;
        n2 -= c;
        test_queue<kPrecise>(q, best, n2, c, a.grid, cells, items, sph, lane);
        if (!flush) break;
      }
      if (flush) break;
      }  // resume the steps after a walk
      __syncwarp();

      const uint32_t key = best.key[lane];
      bool overflowed = false;
      int steps_taken = a.n_steps;
      if (active && key != 0xffffffffu) {
        steps_taken = (int)(key >> 16);
        const PhotonInit in = init_photon_again<kPrecise>(a, s, plo, phi);
        const float wl = in.wl;
        const float3 idir = in.dir;
        const float t0 = in.t0;
        const float4 med = in.med;
        const float3 hpos = make_float3(best.hx[lane], best.hy[lane], best.hz[lane]);
        const float3 hdir = make_float3(best.ox[lane], best.oy[lane], best.oz[lane]);
        const float hdist = best.dist[lane];
        const double time = (double)t0 + (double)hdist / (double)med.y;
        const float abs_w = f_exp<kPrecise>(-f_div<kPrecise>(hdist, med.z));
        if (a.hist) {
          // arrival-time histogram of this source, weighted by absorption
          const float tres = (float)(time - (double)__ldg(a.hist_tgeo + s));
          const float u = log10f(fmaxf(tres + a.hist_t_offset, 1e-30f));
          const int bin =
              min(max((int)floorf((u - a.hist_log_lo) * a.hist_inv_log_width), 0), a.hist_bins - 1);
          float* row = a.hist + (size_t)s * (size_t)(a.hist_bins + 1);
          atomicAdd(row, abs_w);
          atomicAdd(row + 1 + bin, abs_w);
          atomicAdd(u64(&a.counters->n_hits), 1ull);
        } else {
          record_hit(a, hpos, wl, hdir, hdist, idir, abs_w, time, p, (int)(key & 0xffffu) + 1,
                     steps_taken, s, &overflowed);
        }
      }
      if (active) {
        steps_acc += (unsigned long long)steps_taken;
        if (!overflowed) sim_acc += 1;
      }
    }
  }

  // One atomic per warp for the photon and step counters.
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    steps_acc += __shfl_xor_sync(0xffffffffu, steps_acc, o);
    sim_acc += __shfl_xor_sync(0xffffffffu, sim_acc, o);
  }
  if (lane == 0) {
    atomicAdd(u64(&a.counters->photon_steps), steps_acc);
    atomicAdd(u64(&a.counters->n_ph_sim), sim_acc);
  }
}

template <bool P, bool S, bool Sh = false>
const void* kernel_ptr() {
  return reinterpret_cast<const void*>(&propagate_kernel<P, S, Sh>);
}

}  // namespace
}  // namespace pp
