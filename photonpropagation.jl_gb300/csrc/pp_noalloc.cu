// pp_noalloc.cu -- a propagation entry point that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs while another framework
// owns the device memory through its own pooling allocator (a Julia CUDA.jl
// memory pool, a caching allocator that must see every allocation), or
// services that forbid allocation after start-up so that memory use stays
// fixed.  For them
// pp_propagate_static runs the propagation with every piece of scratch memory
// (device copies of the tables, the culling grid and its build buffers, the
// safety field, the work queue and the counters) carved out of one
// file-scope device array of PP_STATIC_SCRATCH_BYTES bytes.  The caller
// passes the inputs (host arrays) and the output hit buffer (device memory).
//
// Properties a caller must know:
//   * the array is part of this library's device image, so every GPU that
//     loads the library holds PP_STATIC_SCRATCH_BYTES until the process exits;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, once per device, with that device current); make
//     that first call before any stream capture begins;
//   * every call copies its inputs from host memory, reads the grid totals
//     and the counters back to the host and synchronises `stream` before it
//     returns, so a call cannot itself be recorded by stream capture;
//   * every call shares the one array and keeps the last call's contents, so
//     calls that overlap on the GPU (several host threads or streams at once)
//     race: serialise them;
//   * inputs whose scratch would exceed the array are rejected with
//     PP_ERR_INVALID and a message naming the limit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "pp_internal.h"

namespace {

static __device__ __align__(256) unsigned char g_static_scratch[PP_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

int fail(int code, const std::string& m) { return pp::report_error(code, m); }

int cuda_fail(cudaError_t e, const char* what) {
  return fail(PP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                               cudaGetErrorString(e) + ")");
}

// Device address of the scratch array on the current device, looked up once.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(PP_ERR_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return PP_OK;
}

// Bump allocator over the scratch array (256-byte aligned regions).
struct Arena {
  unsigned char* base;
  size_t used = 0;
  bool overflow = false;
  template <class T>
  T* take(size_t count) {
    const size_t off = (used + 255) & ~(size_t)255;
    const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    if (off + bytes > PP_STATIC_SCRATCH_BYTES) {
      overflow = true;
      return nullptr;
    }
    used = off + bytes;
    return reinterpret_cast<T*>(base + off);
  }
};

long long scaled_photons(long long photons, float scaling) {
  const float x = (float)photons * scaling;
  if (!(x > 0.0f)) return 0;
  return (long long)floorf(x);
}

// Grid and safety-field shapes from the host copy of the targets, with the
// same box, automatic cell sizes and limits as pp_set_targets.
void grid_shape(const pp_sphere* t, int n, float cell_size, pp::GridDev* g) {
  *g = pp::GridDev{};
  if (n <= 0) {
    for (int a = 0; a < 3; ++a) {
      g->lo[a] = 0.0f; g->hi[a] = 1.0f; g->cell[a] = 1.0f; g->inv_cell[a] = 1.0f; g->dims[a] = 1;
    }
    g->n_cells = 1;
    return;
  }
  float bb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int i = 0; i < n; ++i) {
    const float r = t[i].radius + pp::kGridMargin;
    for (int a = 0; a < 3; ++a) {
      bb[a] = std::min(bb[a], t[i].position[a] - r);
      bb[3 + a] = std::max(bb[3 + a], t[i].position[a] + r);
    }
  }
  double ext[3], vol = 1.0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = std::max(1e-3, (double)bb[3 + a] - (double)bb[a]);
    vol *= ext[a];
  }
  double h = cell_size;
  if (!(h > 0.0)) h = std::cbrt(vol / (16.0 * n));
  for (int guard = 0; guard < 64; ++guard) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::max(1.0, std::ceil(ext[a] / h));
    if (cells <= 4.0 * 1024 * 1024) break;
    h *= 1.25;
  }
  g->n_cells = 1;
  for (int a = 0; a < 3; ++a) {
    g->dims[a] = (int)std::max(1.0, std::ceil(ext[a] / h));
    g->lo[a] = bb[a];
    g->cell[a] = (float)h;
    g->inv_cell[a] = (float)(1.0 / h);
    g->hi[a] = (float)((double)bb[a] + g->dims[a] * h);
    g->n_cells *= g->dims[a];
  }
}

void safety_shape(const pp::GridDev& g, pp::SafetyDev* s) {
  *s = pp::SafetyDev{};
  double ext[3], vol = 1.0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = std::max(1e-6, (double)g.hi[a] - (double)g.lo[a]);
    vol *= ext[a];
  }
  double h = std::max(1e-3, std::cbrt(vol / 32768.0));
  for (int guard = 0; guard < 64; ++guard) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::max(1.0, std::ceil(ext[a] / h));
    if (cells <= 16.0 * 1024 * 1024) break;
    h *= 1.25;
  }
  s->n_cells = 1;
  for (int a = 0; a < 3; ++a) {
    s->dims[a] = (int)std::max(1.0, std::ceil(ext[a] / h));
    s->lo[a] = g.lo[a];
    s->hi[a] = (float)((double)g.lo[a] + s->dims[a] * h);
    s->n_cells *= s->dims[a];
  }
  s->cell = (float)h;
  s->inv_cell = (float)(1.0 / h);
  s->bytes = (uint32_t)(((size_t)s->n_cells + 15) & ~(size_t)15);
  s->set_derived();
}

// Upper bound of the grid's item count from the host copy of the targets.
size_t item_bound(const pp_sphere* t, int n, const pp::GridDev& g) {
  size_t total = 0;
  for (int i = 0; i < n; ++i) {
    size_t c = 1;
    for (int a = 0; a < 3; ++a) {
      const float r = t[i].radius + pp::kGridMargin;
      const int lo = (int)std::floor((t[i].position[a] - r - g.lo[a]) * g.inv_cell[a]) - 1;
      const int hi = (int)std::floor((t[i].position[a] + r - g.lo[a]) * g.inv_cell[a]) + 1;
      c *= (size_t)(std::min(hi, g.dims[a] - 1) - std::max(lo, 0) + 1);
    }
    total += c;
  }
  return total;
}

}  // namespace

extern "C" PP_API int pp_propagate_static(
    const pp_medium* medium, const float* spectrum_knots, int32_t n_spectrum,
    float mono_wavelength, const float* track_quantiles, int32_t n_track,
    const pp_sphere* targets, int32_t n_targets, float cell_size, const pp_source* sources,
    int32_t n_src, int64_t seed, int32_t n_steps, float photon_scaling, pp_hit_record* d_hits,
    int64_t capacity, pp_counters* counters, void* stream_ptr) {
  // ---- validation (same rules as the context-based entry points) ----
  if (!medium || !counters) return fail(PP_ERR_INVALID, "null argument");
  if (medium->n_knots < 2 || !(medium->wl_step > 0.0f) || !medium->scattering_length ||
      !medium->group_velocity || !medium->absorption_length || !medium->phase_refractive_index)
    return fail(PP_ERR_INVALID, "medium needs n_knots >= 2, wl_step > 0 and four tables");
  pp::PhaseDev phase{};
  if (const char* why = pp::make_phase(medium, &phase)) return fail(PP_ERR_INVALID, why);
  if (n_spectrum < 0 || (n_spectrum > 0 && !spectrum_knots) ||
      (n_spectrum == 0 && !(mono_wavelength > 0.0f)))
    return fail(PP_ERR_INVALID, "spectrum: pass knots or a positive monochromatic wavelength");
  if (n_targets < 0 || n_targets > 65535 || (n_targets > 0 && !targets))
    return fail(PP_ERR_INVALID, "targets: 0..65535 spheres");
  if (n_src < 0 || (n_src > 0 && !sources)) return fail(PP_ERR_INVALID, "bad source list");
  if (n_steps < 1 || n_steps > 65535) return fail(PP_ERR_INVALID, "n_steps must be in [1, 65535]");
  if (!(photon_scaling >= 0.0f) || capacity < 0 || (capacity > 0 && !d_hits) ||
      ((uintptr_t)d_hits & 15u))
    return fail(PP_ERR_INVALID, "bad scaling, capacity or hit buffer");
  bool needs_track = false;
  for (int i = 0; i < n_src; ++i) {
    const int k = sources[i].kind;
    if (k < 0 || k >= PP_SRC_KIND_COUNT || sources[i].photons < 0)
      return fail(PP_ERR_INVALID, "source " + std::to_string(i) + " is invalid");
    if ((k == PP_SRC_EXTENDED_CHERENKOV || k == PP_SRC_EXTENDED_CHERENKOV_NOSMEAR) &&
        !(sources[i].long_a > 0.0f && sources[i].long_b > 0.0f))
      return fail(PP_ERR_INVALID, "source " + std::to_string(i) + ": bad longitudinal parameters");
    const bool track = k == PP_SRC_EXTENDED_CHERENKOV || k == PP_SRC_POINTLIKE_CHERENKOV ||
                       k == PP_SRC_CHERENKOV_TRACK;
    if (track && sources[i].smear_table != 0)  // one table here
      return fail(PP_ERR_INVALID, "source " + std::to_string(i) + ": smear_table must be 0");
    needs_track |= track;
  }
  if (needs_track && (n_track < 2 || !track_quantiles))
    return fail(PP_ERR_INVALID, "Cherenkov emitters need the track-direction table");
  for (int i = 0; i < n_targets; ++i)
    if (!(targets[i].radius > 0.0f)) return fail(PP_ERR_INVALID, "target radius must be > 0");

  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(PP_ERR_NO_DEVICE, "no CUDA device available");
  }
  unsigned char* base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc != PP_OK) return rc;
  cudaStream_t stream = (cudaStream_t)stream_ptr;
  int dev = 0, num_sms = 0;
  cudaError_t ae = cudaGetDevice(&dev);
  if (ae == cudaSuccess) ae = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
  if (ae != cudaSuccess) return cuda_fail(ae, "SM count");
  if (num_sms < 1) return fail(PP_ERR_CUDA, "device reports no multiprocessors");

  // ---- host-side shapes and the work queue ----
  pp::GridDev gshape;
  grid_shape(targets, n_targets, cell_size, &gshape);
  pp::SafetyDev sshape;
  safety_shape(gshape, &sshape);
  const int ppt = 8, block = 1024;
  const long long chunk = 32LL * ppt;
  std::vector<unsigned long long> prefix(n_src + 1, 0);
  std::vector<long long> nph(std::max(n_src, 1), 0);
  for (int i = 0; i < n_src; ++i) {
    nph[i] = scaled_photons(sources[i].photons, photon_scaling);
    prefix[i + 1] = prefix[i] + (unsigned long long)((nph[i] + chunk - 1) / chunk);
  }
  std::vector<float4> table(medium->n_knots);
  for (int i = 0; i < medium->n_knots; ++i) {
    table[i] = make_float4(medium->scattering_length[i], medium->group_velocity[i],
                           medium->absorption_length[i], medium->phase_refractive_index[i]);
    if (!(table[i].x > 0.0f) || !(table[i].y > 0.0f) || !(table[i].z > 0.0f) || !(table[i].w > 0.0f))
      return fail(PP_ERR_INVALID, "medium table entries must be positive");
  }

  // the fast kernel's tabulated ES inverse CDF, as pp_set_medium makes it
  std::vector<float2> es;
  if (phase.kind == PP_PHASE_HG_ES && medium->hg_weight < 1.0f) {
    es.resize(pp::kEsTable);
    pp::make_es_table(phase.es_b, es.data());
  }

  // ---- carve the scratch ----
  Arena ar{base};
  float4* d_medium = ar.take<float4>(table.size());
  float2* d_es = ar.take<float2>(std::max<size_t>(es.size(), 1));
  float* d_spec = ar.take<float>(std::max(n_spectrum, 1));
  float* d_track = ar.take<float>(std::max(n_track, 1));
  pp_sphere* d_targets = ar.take<pp_sphere>(std::max(n_targets, 1));
  pp_source* d_sources = ar.take<pp_source>(std::max(n_src, 1));
  unsigned long long* d_prefix = ar.take<unsigned long long>(n_src + 1);
  long long* d_photons = ar.take<long long>(std::max(n_src, 1));
  pp_counters* d_ctr = ar.take<pp_counters>(1);
  unsigned* d_counts = ar.take<unsigned>(gshape.n_cells);
  unsigned* d_start = ar.take<unsigned>(gshape.n_cells);
  unsigned* d_cursor = ar.take<unsigned>(gshape.n_cells);
  unsigned* d_totals = ar.take<unsigned>(2);
  const size_t blob_cap = (((size_t)gshape.n_cells * 4 + 15) & ~(size_t)15) +
                          ((item_bound(targets, n_targets, gshape) * 2 + 15) & ~(size_t)15) + 16 +
                          (size_t)n_targets * sizeof(float4);
  unsigned char* d_blob = ar.take<unsigned char>(blob_cap);
  unsigned char* d_field = ar.take<unsigned char>(sshape.bytes);
  if (ar.overflow)
    return fail(PP_ERR_INVALID, "inputs need more scratch than the " +
                                    std::to_string(PP_STATIC_SCRATCH_BYTES >> 20) +
                                    " MiB static array holds (fewer targets, sources or table knots)");

  // ---- inputs into the scratch (copies only; nothing is allocated) ----
  auto h2d = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream) : cudaSuccess;
  };
  cudaError_t e = h2d(d_medium, table.data(), table.size() * sizeof(float4));
  if (e == cudaSuccess && !es.empty()) e = h2d(d_es, es.data(), es.size() * sizeof(float2));
  if (e == cudaSuccess && n_spectrum > 0) e = h2d(d_spec, spectrum_knots, n_spectrum * sizeof(float));
  if (e == cudaSuccess && n_track > 0 && track_quantiles)
    e = h2d(d_track, track_quantiles, n_track * sizeof(float));
  if (e == cudaSuccess && n_targets > 0) e = h2d(d_targets, targets, n_targets * sizeof(pp_sphere));
  if (e == cudaSuccess && n_src > 0) e = h2d(d_sources, sources, n_src * sizeof(pp_source));
  if (e == cudaSuccess) e = h2d(d_prefix, prefix.data(), prefix.size() * sizeof(unsigned long long));
  if (e == cudaSuccess && n_src > 0) e = h2d(d_photons, nph.data(), n_src * sizeof(long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ctr, 0, sizeof(pp_counters), stream);
  if (e != cudaSuccess) return cuda_fail(e, "copy inputs to the static scratch");

  // ---- culling grid and safety field, built in the scratch ----
  std::string err;
  pp::GridDev grid;
  long long n_items = 0;
  if (pp::build_grid_into(d_targets, n_targets, gshape, d_counts, d_start, d_cursor, d_totals,
                          d_blob, blob_cap, stream, &grid, &n_items, &err) != 0)
    return fail(PP_ERR_INVALID, "grid: " + err);
  if (pp::build_safety_into(d_targets, n_targets, sshape, d_field, stream, &err) != 0)
    return fail(PP_ERR_CUDA, err);

  // ---- launch (fast variant, default launch shape) ----
  pp::LaunchArgs a{};
  a.sources = d_sources;
  a.chunk_prefix = d_prefix;
  a.src_photons = d_photons;
  a.total_chunks = prefix[n_src];
  a.n_src = n_src;
  a.chunk_photons = (int)chunk;
  a.blob = d_blob;
  a.grid = grid;
  a.safety = d_field;
  a.sgrid = sshape;
  a.medium = d_medium;
  a.n_medium = medium->n_knots;
  a.med_wl_min = medium->wl_min;
  a.med_inv_step = 1.0f / medium->wl_step;
  phase.es_table = es.empty() ? nullptr : d_es;
  a.phase = phase;
  a.spectrum = n_spectrum > 0 ? d_spec : nullptr;
  a.n_spectrum = n_spectrum;
  a.mono_wavelength = mono_wavelength;
  a.track = needs_track ? d_track : nullptr;
  a.n_track = n_track;
  a.set_seed((uint64_t)seed);
  a.n_steps = n_steps;
  a.hits = d_hits;
  a.capacity = (unsigned long long)capacity;
  a.counters = d_ctr;
  a.wait_limit_ns = 2000000000ull;
  if (a.total_chunks > 0) {
    const bool smem = pp::propagate_smem_bytes(grid.blob_bytes, sshape.bytes, true, block, nullptr,
                                               nullptr) <= pp::smem_budget(block);
    e = pp::launch_propagate(a, block, 0, false, smem, num_sms, stream, nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "launch propagate kernel");
  }
  pp_counters c{};
  e = cudaMemcpyAsync(&c, d_ctr, sizeof(c), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(e, "propagate (static scratch)");
  *counters = c;
  if (c.err_flags & PP_FLAG_TIMEOUT)
    return fail(PP_ERR_TIMEOUT, "a bounded device wait (TMA staging) timed out");
  if ((c.err_flags & PP_FLAG_OVERFLOW) || (long long)c.n_hits > capacity)
    return fail(PP_ERR_OVERFLOW, "hit buffer overflow: " + std::to_string(c.n_hits) +
                                     " hits, capacity " + std::to_string(capacity));
  return PP_OK;
}
