// pp_pmt.cu -- photon hits -> PMT hits on the device: the detection step that
// follows propagation in the reference (make_hits_from_photons and
// calc_pe_weight!, src/processing.jl:88-205), one thread per hit record.
//
// For a POM (src/pom.jl:246-305, POMAcceptance): with rel = (hit - centre) / r,
// for each of the 16 PMTs (unit vector p_i, group g_i)
//   pt_i  = acos(clamp(rel . p_i, -1, 1))
//   w_i   = Rayleigh_{sigma_g}(pt_i) / (sin(pt_i) / 2)   (0 where sin(pt_i) = 0)
//   prob_i = w_i * acc_g(wavelength) / 8
// the photon is detected when u1 < sum_i prob_i, by PMT i chosen with
// probability prob_i / sum (the first i whose running sum reaches u2 * sum).
// acc_g and the relative quantum efficiency are linear interpolations that
// are 0 outside their tables (Interpolations.jl, extrapolation_bc = 0).
// For a homogeneous module (src/detection.jl:57-84) the photon is detected
// when u1 < active_area / (4 pi r^2), as PMT 1.
// For a DOM (src/dom.jl:96-134) it is detected, as PMT 1, when
// u1 * polymax < poly(cos zenith of its direction) and u2 < wl_acc(wavelength)
// (the second test only when the model asks for the wavelength acceptance).
// For a multi-PMT module (src/detection.jl:90-131) it is detected when
// u1 <= sum_i max(dir . q_i, 0) * pmt_area / (pi r^2) (q_i the PMT axes in the
// module frame), by the PMT that StatsBase's weighted sample picks for u2 over
// the weights w_i = -(rel . p_i) (p_i the oriented axes): the first i whose
// running sum reaches u2 * sum_i w_i, else the last.
// u1, u2 are Philox4x32-10 uniforms of counter (hit index, 0x504d5400, 0),
// key = seed, so a CPU restatement can replay every decision (up to the
// rounding of the arithmetic: sin(pt) is evaluated as sqrt(1 - cos^2 pt),
// the Gaussian factor by exp2f).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "pp_device.cuh"
#include "pp_internal.h"

namespace {

constexpr int kPomPmts = 16;
constexpr uint32_t kPmtStream = 0x504d5400u;  // Philox counter word that tags this stream

struct PmtArgs {
  const pp_hit_record* rec;
  long long n;
  const pp_pmt_target* targets;
  int n_targets;
  const pp_pom_model* pom;  // device copies, each may be null
  const pp_dom_model* dom;
  const pp_multipmt_model* mpmt;
  uint32_t key0, key1;
  int32_t* pmt_id;
  float* qe_weight;         // may be null
};

// Linear interpolation on ascending knots, 0 outside [x[0], x[n-1]].
__device__ __forceinline__ float interp0(const float* x, const float* y, int n, float v) {
  if (n < 2 || !(v >= x[0]) || !(v <= x[n - 1])) return 0.0f;
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (x[mid] <= v) lo = mid;
    else hi = mid;
  }
  const float t = (v - x[lo]) / (x[hi] - x[lo]);
  return fmaf(t, y[hi] - y[lo], y[lo]);
}

template <class T>
__device__ __forceinline__ void stage(T* dst, const T* src) {
  static_assert(sizeof(T) % 4 == 0, "word copy");
  if (!src) return;
  const int* s = reinterpret_cast<const int*>(src);
  int* d = reinterpret_cast<int*>(dst);
  for (int w = threadIdx.x; w < (int)(sizeof(T) / 4); w += blockDim.x) d[w] = s[w];
}

// The models in shared memory (staged once per block; the grid strides).
__global__ void __launch_bounds__(256) pmt_kernel(const PmtArgs a) {
  __shared__ pp_pom_model sm;
  __shared__ pp_dom_model sdom;
  __shared__ pp_multipmt_model smp;
  stage(&sm, a.pom);
  stage(&sdom, a.dom);
  stage(&smp, a.mpmt);
  __syncthreads();
  // Rayleigh(pt; sigma) = pt / sigma^2 * 2^(pt^2 * (-log2(e) / (2 sigma^2))), per group
  const float inv_s2_1 = 1.0f / (sm.sigma_group1 * sm.sigma_group1);
  const float inv_s2_2 = 1.0f / (sm.sigma_group2 * sm.sigma_group2);
  const float e2_1 = -0.72134752044448170368f * inv_s2_1;  // -log2(e) / 2
  const float e2_2 = -0.72134752044448170368f * inv_s2_2;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a.n;
       i += (long long)gridDim.x * blockDim.x) {
    const float4* r = reinterpret_cast<const float4*>(a.rec + i);
    // the record's first 32 bytes: position, wavelength; direction, module
    const float4 pw = __ldg(r);
    const float4 dw = __ldg(r + 1);
    const int module = __float_as_int(dw.w);  // 1-based
    int id = 0;
    float qe = 0.0f;
    if (module >= 1 && module <= a.n_targets) {
      const pp_pmt_target t = a.targets[module - 1];
      const uint4 u = ppdev::philox(make_uint4((uint32_t)i, (uint32_t)((unsigned long long)i >> 32),
                                            kPmtStream, 0u),
                                 a.key0, a.key1);
      const float u1 = ppdev::u01(u.x), u2 = ppdev::u01(u.y);
      if (t.kind == PP_PMT_HOMOGENEOUS) {
        const float frac = t.active_area / (4.0f * 3.14159265358979f * t.radius * t.radius);
        id = u1 < frac ? 1 : 0;
        qe = 1.0f;
      } else if (t.kind == PP_PMT_POM && a.pom) {
        const pp_pom_model& m = sm;
        const float inv_r = 1.0f / t.radius;
        const float rx = (pw.x - t.position[0]) * inv_r;
        const float ry = (pw.y - t.position[1]) * inv_r;
        const float rz = (pw.z - t.position[2]) * inv_r;
        const float acc1 = interp0(m.acc_wavelength, m.acc_group1, m.n_acc, pw.w);
        const float acc2 = interp0(m.acc_wavelength, m.acc_group2, m.n_acc, pw.w);
        float prob[kPomPmts];
        float total = 0.0f;
#pragma unroll
        for (int k = 0; k < kPomPmts; ++k) {
          const float c = fminf(fmaxf(rx * m.pmt_dir[k][0] + ry * m.pmt_dir[k][1] +
                                          rz * m.pmt_dir[k][2], -1.0f), 1.0f);
          const float pt = acosf(c);
          const bool g1 = m.pmt_group[k] == 1;
          const float s = sqrtf(fmaxf(1.0f - c * c, 0.0f));  // sin(acos(c)) for pt in [0, pi]
          const float pdf = pt * (g1 ? inv_s2_1 : inv_s2_2) * exp2f(pt * pt * (g1 ? e2_1 : e2_2));
          // w / 8 = pdf / (s / 2) / 8 = pdf / (4 s)
          prob[k] = s != 0.0f ? __fdividef(pdf, 4.0f * s) * (g1 ? acc1 : acc2) : 0.0f;
          total += prob[k];
        }
        if (u1 < total) {
          const float target = u2 * total;
          float cum = 0.0f;
          id = kPomPmts;
#pragma unroll
          for (int k = 0; k < kPomPmts; ++k) {
            cum += prob[k];
            if (cum >= target) {
              id = k + 1;
              break;
            }
          }
        }
        qe = interp0(m.qe_wavelength, m.qe, m.n_qe, pw.w);
      } else if (t.kind == PP_PMT_DOM && a.dom) {
        const pp_dom_model& m = sdom;
        const float cz = dw.x * m.zenith_axis[0] + dw.y * m.zenith_axis[1] + dw.z * m.zenith_axis[2];
        float poly = 0.0f;
        for (int k = m.n_poly - 1; k >= 0; --k) poly = fmaf(poly, cz, m.poly[k]);
        const bool ang = u1 * m.polymax < poly;
        const bool wl = !m.apply_wl_acceptance || u2 < interp0(m.wl, m.wl_acc, m.n_wl, pw.w);
        id = ang && wl ? 1 : 0;
        qe = 1.0f;
      } else if (t.kind == PP_PMT_MULTIPMT && a.mpmt) {
        const pp_multipmt_model& m = smp;
        float proj = 0.0f;
        for (int k = 0; k < m.n_pmt; ++k) {
          const float c = dw.x * m.pmt_dir_module[k][0] + dw.y * m.pmt_dir_module[k][1] +
                          dw.z * m.pmt_dir_module[k][2];
          if (c > 0.0f) proj += c;
        }
        const float prob = proj * m.pmt_area / (3.14159265358979f * t.radius * t.radius);
        if (u1 <= prob) {
          const float inv_r = 1.0f / t.radius;
          const float rx = (pw.x - t.position[0]) * inv_r;
          const float ry = (pw.y - t.position[1]) * inv_r;
          const float rz = (pw.z - t.position[2]) * inv_r;
          float wsum = 0.0f;
          for (int k = 0; k < m.n_pmt; ++k)
            wsum -= rx * m.pmt_dir[k][0] + ry * m.pmt_dir[k][1] + rz * m.pmt_dir[k][2];
          const float target = u2 * wsum;
          int j = 0;
          float cw = -(rx * m.pmt_dir[0][0] + ry * m.pmt_dir[0][1] + rz * m.pmt_dir[0][2]);
          while (cw < target && j < m.n_pmt - 1) {
            ++j;
            cw -= rx * m.pmt_dir[j][0] + ry * m.pmt_dir[j][1] + rz * m.pmt_dir[j][2];
          }
          id = j + 1;
        }
        qe = interp0(m.qe_wavelength, m.qe, m.n_qe, pw.w);
      }
    }
    a.pmt_id[i] = id;
    if (a.qe_weight) a.qe_weight[i] = qe;
  }
}

__global__ void tres_kernel(const pp_hit_record* __restrict__ rec, long long n,
                            const double* __restrict__ tgeo, int n_targets, double t0,
                            double* __restrict__ tres) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int module = rec[i].module_index;  // 1-based
    tres[i] = module >= 1 && module <= n_targets ? rec[i].time - tgeo[module - 1] - t0
                                                 : __longlong_as_double(0x7ff8000000000000ll);
  }
}

}  // namespace

extern "C" {

PP_API int pp_time_residuals(const pp_hit_record* d_records, int64_t n, const double* tgeo,
                             int32_t n_targets, double t0, double* d_tres, void* stream) {
  if (n < 0 || (n > 0 && (!d_records || !d_tres)) || n_targets < 0 || (n_targets > 0 && !tgeo))
    return pp::report_error(PP_ERR_INVALID, "pp_time_residuals: bad arguments");
  if (n == 0) return PP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  double* d_tg = nullptr;
  const size_t tb = sizeof(double) * (size_t)(n_targets > 0 ? n_targets : 1);
  cudaError_t e = cudaMallocAsync((void**)&d_tg, tb, s);
  if (e == cudaSuccess && n_targets > 0)
    e = cudaMemcpyAsync(d_tg, tgeo, sizeof(double) * n_targets, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = std::min<long long>((n + 255) / 256, (long long)sms * 8);
    tres_kernel<<<(unsigned)blocks, 256, 0, s>>>(d_records, n, d_tg, n_targets, t0, d_tres);
    e = cudaGetLastError();
  }
  if (d_tg) cudaFreeAsync(d_tg, s);
  if (e != cudaSuccess)
    return pp::report_error(PP_ERR_CUDA, std::string("pp_time_residuals: ") + cudaGetErrorString(e));
  return PP_OK;
}

PP_API int pp_make_hits_from_photons_models(const pp_hit_record* d_records, int64_t n,
                                            const pp_pmt_target* targets, int32_t n_targets,
                                            const pp_detection_models* models, int64_t seed,
                                            int32_t* d_pmt_id, float* d_qe_weight, void* stream) {
  static const char* kWho = "pp_make_hits_from_photons: ";
  if (n < 0 || (n > 0 && (!d_records || !d_pmt_id)) || n_targets < 0 ||
      (n_targets > 0 && !targets))
    return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "bad arguments");
  const pp_pom_model* pom = models ? models->pom : nullptr;
  const pp_dom_model* dom = models ? models->dom : nullptr;
  const pp_multipmt_model* mp = models ? models->multipmt : nullptr;
  if (pom && (pom->n_acc < 2 || pom->n_acc > PP_POM_MAX_KNOTS || pom->n_qe < 2 ||
              pom->n_qe > PP_POM_MAX_KNOTS))
    return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "bad POM tables");
  if (dom && (dom->n_poly < 1 || dom->n_poly > PP_DOM_MAX_POLY || dom->n_wl < 2 ||
              dom->n_wl > PP_POM_MAX_KNOTS))
    return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "bad DOM tables");
  if (mp && (mp->n_pmt < 1 || mp->n_pmt > PP_MULTIPMT_MAX_PMTS || mp->n_qe < 2 ||
             mp->n_qe > PP_POM_MAX_KNOTS))
    return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "bad multi-PMT tables");
  for (int i = 0; i < n_targets; ++i) {
    const int k = targets[i].kind;
    if (k != PP_PMT_HOMOGENEOUS && k != PP_PMT_POM && k != PP_PMT_DOM && k != PP_PMT_MULTIPMT)
      return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "unknown module kind");
    if ((k == PP_PMT_POM && !pom) || (k == PP_PMT_DOM && !dom) || (k == PP_PMT_MULTIPMT && !mp))
      return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "module without its model");
    if (!(targets[i].radius > 0.0f))
      return pp::report_error(PP_ERR_INVALID, std::string(kWho) + "target radius <= 0");
  }
  if (n == 0) return PP_OK;
  cudaStream_t s = (cudaStream_t)stream;
  // one staging allocation: targets, then each model at a 16-byte boundary
  auto up16 = [](size_t b) { return (b + 15) & ~size_t(15); };
  const size_t tb = up16(sizeof(pp_pmt_target) * (size_t)(n_targets > 0 ? n_targets : 1));
  const size_t ob_pom = tb, ob_dom = ob_pom + (pom ? up16(sizeof(pp_pom_model)) : 0);
  const size_t ob_mp = ob_dom + (dom ? up16(sizeof(pp_dom_model)) : 0);
  const size_t total = ob_mp + (mp ? up16(sizeof(pp_multipmt_model)) : 0);
  unsigned char* buf = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&buf, total, s);
  if (e == cudaSuccess && n_targets > 0)
    e = cudaMemcpyAsync(buf, targets, sizeof(pp_pmt_target) * n_targets, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && pom)
    e = cudaMemcpyAsync(buf + ob_pom, pom, sizeof(pp_pom_model), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && dom)
    e = cudaMemcpyAsync(buf + ob_dom, dom, sizeof(pp_dom_model), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && mp)
    e = cudaMemcpyAsync(buf + ob_mp, mp, sizeof(pp_multipmt_model), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) {
    if (buf) cudaFreeAsync(buf, s);
    return pp::report_error(PP_ERR_CUDA, std::string(kWho) + cudaGetErrorString(e));
  }
  PmtArgs a{};
  a.rec = d_records;
  a.n = n;
  a.targets = reinterpret_cast<const pp_pmt_target*>(buf);
  a.n_targets = n_targets;
  a.pom = pom ? reinterpret_cast<const pp_pom_model*>(buf + ob_pom) : nullptr;
  a.dom = dom ? reinterpret_cast<const pp_dom_model*>(buf + ob_dom) : nullptr;
  a.mpmt = mp ? reinterpret_cast<const pp_multipmt_model*>(buf + ob_mp) : nullptr;
  a.key0 = (uint32_t)(uint64_t)seed;
  a.key1 = (uint32_t)((uint64_t)seed >> 32);
  a.pmt_id = d_pmt_id;
  a.qe_weight = d_qe_weight;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long blocks = std::min<long long>((n + 255) / 256, (long long)sms * 8);
  pmt_kernel<<<(unsigned)blocks, 256, 0, s>>>(a);
  e = cudaGetLastError();
  cudaFreeAsync(buf, s);
  if (e != cudaSuccess)
    return pp::report_error(PP_ERR_CUDA, std::string(kWho) + cudaGetErrorString(e));
  return PP_OK;
}

PP_API int pp_make_hits_from_photons(const pp_hit_record* d_records, int64_t n,
                                     const pp_pmt_target* targets, int32_t n_targets,
                                     const pp_pom_model* pom, int64_t seed, int32_t* d_pmt_id,
                                     float* d_qe_weight, void* stream) {
  const pp_detection_models models{pom, nullptr, nullptr};
  return pp_make_hits_from_photons_models(d_records, n, targets, n_targets, &models, seed,
                                          d_pmt_id, d_qe_weight, stream);
}

}  // extern "C"
