// pp_abi.cu -- the C ABI (include/pp_gb300.h): contexts, device tables, the
// synchronous drop-in propagate call, asynchronous and graph-replayed
// launches, and the launch autotuner.
//
// Host-side counterpart of run_photon_prop_no_local_cache!
// (PhotonPropagation.jl v0.9.3, src/photon_prop_cuda.jl:889-959).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "pp_internal.h"

using pp::GridDev;
using pp::LaunchArgs;

namespace {

thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  return set_error(PP_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define PP_CUDA(call, what)                  \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) return cuda_error(e_, what); \
  } while (0)

// Makes ctx->device current for the scope of one ABI call.
struct DeviceScope {
  int prev = -1;
  explicit DeviceScope(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    if (prev != dev) cudaSetDevice(dev);
  }
  ~DeviceScope() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

bool is_device_pointer(const void* p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

long long source_photons(long long photons, float scaling) {
  // Int64 * Float32 promotes to Float32 (src/photon_prop_cuda.jl:456).
  const float x = (float)photons * scaling;
  if (!(x > 0.0f)) return 0;
  return (long long)floorf(x);
}

bool kind_uses_track(int kind) {
  return kind == PP_SRC_EXTENDED_CHERENKOV || kind == PP_SRC_POINTLIKE_CHERENKOV ||
         kind == PP_SRC_CHERENKOV_TRACK;
}

}  // namespace

namespace pp {
// Error reporting for entry points defined in other translation units.
int report_error(int code, const std::string& message) {
  g_last_error = message;
  return code;
}
}  // namespace pp

struct GraphKey {
  long long seed = 0;
  int n_steps = 0;
  const void* hits = nullptr;
  long long capacity = 0;
  const void* counters = nullptr;
  cudaStream_t stream = nullptr;
  unsigned long long version = 0;
  bool operator==(const GraphKey& o) const {
    return seed == o.seed && n_steps == o.n_steps && hits == o.hits && capacity == o.capacity &&
           counters == o.counters && stream == o.stream && version == o.version;
  }
};

struct pp_ctx {
  int device = 0;
  int num_sms = 0;
  int chunk_photons = 256;  // photons per queued chunk (build_queue)
  cudaStream_t stream = nullptr;
  // recorded after every launch on the caller's stream: setters wait on it
  // before they overwrite device inputs that a launch in flight still reads
  cudaEvent_t inflight = nullptr;
  unsigned long long version = 1;

  // medium
  float4* d_medium = nullptr;
  int n_medium = 0;
  float med_wl_min = 0.0f, med_inv_step = 0.0f;
  pp::PhaseDev phase{};
  float2* d_es_table = nullptr;  // the phase function's tabulated ES inverse CDF
  bool has_medium = false;

  // spectrum
  float* d_spectrum = nullptr;
  int n_spectrum = 0;
  float mono = 0.0f;
  bool has_spectrum = false;

  // Cherenkov track smear quantiles: n_track_tables tables of n_track knots
  float* d_track = nullptr;
  int n_track = 0;
  int n_track_tables = 0;
  int max_smear_table = 0;  // largest smear_table of the track-using sources

  // targets and grid
  std::vector<pp_sphere> h_targets;
  pp_sphere* d_targets = nullptr;
  float4* d_shapes = nullptr;  // shaped targets (then the sphere list is empty)
  float4* d_loop_spheres = nullptr;  // the sphere list as shape records (target_loop)
  int n_shapes = 0;
  unsigned char* d_blob = nullptr;
  GridDev grid{};
  unsigned char* d_safety = nullptr;
  pp::SafetyDev sgrid{};
  long long n_items = 0;
  bool has_targets = false;

  // sources and work queue
  std::vector<pp_source> h_sources;
  float scaling = 1.0f;
  pp_source* d_sources = nullptr;
  unsigned long long* d_prefix = nullptr;
  long long* d_src_photons = nullptr;
  int n_src = 0;
  int n_src_alloc = 0;
  unsigned long long total_chunks = 0;
  long long total_photons = 0;
  bool has_sources = false;
  bool needs_track = false;

  pp_tuning tuning{1024, 8, 0, 0, 0.0f, 0, 0.0f, 0};

  // scratch of pp_propagate
  pp_hit_record* d_hits = nullptr;
  long long d_hits_cap = 0;
  pp_counters* d_ctr = nullptr;
  pp_hit_record* h_stage = nullptr;
  long long h_stage_cap = 0;

  // cached CUDA graph of pp_launch_graph
  cudaGraphExec_t gexec = nullptr;
  GraphKey gkey{};

  long long last_hits = 0;  // hits held in d_hits from the last pp_propagate
};

namespace {

int build_queue(pp_ctx* ctx) {
  const int n = (int)ctx->h_sources.size();
  std::vector<unsigned long long> prefix(n + 1, 0);
  std::vector<long long> nph(std::max(n, 1), 0);
  long long total = 0;
  for (int i = 0; i < n; ++i) {
    nph[i] = source_photons(ctx->h_sources[i].photons, ctx->scaling);
    total += nph[i];
  }
  // Small workloads: halve the photons per lane and chunk until there are at
  // least two chunks for every warp the GPU holds at once (32 per SM), so
  // that a 1e5-photon call is not run by a tenth of the warps.  Photons draw
  // their random numbers by index, so the chunking changes no result.
  int ppt = ctx->tuning.photons_per_thread;
  const long long resident_warps = 32LL * std::max(ctx->num_sms, 1);
  while (ppt > 1 && total / (32LL * ppt) < 2 * resident_warps) ppt /= 2;
  const long long chunk = 32LL * ppt;
  for (int i = 0; i < n; ++i)
    prefix[i + 1] = prefix[i] + (unsigned long long)((nph[i] + chunk - 1) / chunk);
  ctx->chunk_photons = (int)chunk;
  if (n > ctx->n_src_alloc) {
    cudaFree(ctx->d_sources);
    cudaFree(ctx->d_prefix);
    cudaFree(ctx->d_src_photons);
    ctx->d_sources = nullptr;
    ctx->d_prefix = nullptr;
    ctx->d_src_photons = nullptr;
    ctx->n_src_alloc = 0;
    PP_CUDA(cudaMalloc(&ctx->d_sources, sizeof(pp_source) * n), "cudaMalloc(sources)");
    PP_CUDA(cudaMalloc(&ctx->d_prefix, sizeof(unsigned long long) * (n + 1)), "cudaMalloc(prefix)");
    PP_CUDA(cudaMalloc(&ctx->d_src_photons, sizeof(long long) * n), "cudaMalloc(photons)");
    ctx->n_src_alloc = n;
  }
  if (n > 0) {
    PP_CUDA(cudaMemcpyAsync(ctx->d_sources, ctx->h_sources.data(), sizeof(pp_source) * n,
                            cudaMemcpyHostToDevice, ctx->stream), "upload sources");
    PP_CUDA(cudaMemcpyAsync(ctx->d_prefix, prefix.data(), sizeof(unsigned long long) * (n + 1),
                            cudaMemcpyHostToDevice, ctx->stream), "upload prefix");
    PP_CUDA(cudaMemcpyAsync(ctx->d_src_photons, nph.data(), sizeof(long long) * n,
                            cudaMemcpyHostToDevice, ctx->stream), "upload photon counts");
    PP_CUDA(cudaStreamSynchronize(ctx->stream), "upload sources");
  }
  ctx->n_src = n;
  ctx->total_chunks = prefix[n];
  ctx->total_photons = total;
  ctx->version++;
  return PP_OK;
}

int rebuild_grid(pp_ctx* ctx, float cell_size) {
  cudaFree(ctx->d_blob);
  ctx->d_blob = nullptr;
  std::string err;
  GridDev g{};
  unsigned char* blob = nullptr;
  long long n_items = 0;
  const int n = (int)ctx->h_targets.size();
  if (pp::build_grid(ctx->d_targets, n, cell_size, ctx->stream, &g, &blob, &n_items, &err) != 0)
    return set_error(PP_ERR_INVALID, "pp_set_targets: %s", err.c_str());
  ctx->grid = g;
  ctx->d_blob = blob;
  ctx->n_items = n_items;
  // Safety field over the same box; automatic cell: about 32k cells (32 KiB).
  cudaFree(ctx->d_safety);
  ctx->d_safety = nullptr;
  float hs = ctx->tuning.safety_cell;
  if (!(hs > 0.0f)) {
    double vol = 1.0;
    for (int a = 0; a < 3; ++a) vol *= std::max(1e-6, (double)g.hi[a] - (double)g.lo[a]);
    hs = (float)std::max(1e-3, std::cbrt(vol / 32768.0));
  }
  pp::SafetyDev sg{};
  unsigned char* field = nullptr;
  if (pp::build_safety(ctx->d_targets, n, g, hs, ctx->stream, &sg, &field, &err) != 0)
    return set_error(PP_ERR_CUDA, "pp_set_targets: %s", err.c_str());
  ctx->sgrid = sg;
  ctx->d_safety = field;
  ctx->version++;
  return PP_OK;
}

int check_ready(const pp_ctx* ctx) {
  if (!ctx->has_medium) return set_error(PP_ERR_NOT_READY, "medium not set (pp_set_medium)");
  if (!ctx->has_spectrum)
    return set_error(PP_ERR_NOT_READY, "spectrum not set (pp_set_spectrum / pp_set_monochromatic)");
  if (!ctx->has_targets) return set_error(PP_ERR_NOT_READY, "targets not set (pp_set_targets)");
  if (!ctx->has_sources) return set_error(PP_ERR_NOT_READY, "sources not set (pp_set_sources)");
  if (ctx->needs_track && ctx->n_track < 2)
    return set_error(PP_ERR_NOT_READY,
                     "Cherenkov emitters need the track-direction table (pp_set_track_smear)");
  if (ctx->needs_track && ctx->max_smear_table >= ctx->n_track_tables)
    return set_error(PP_ERR_NOT_READY, "a source uses track-smear table %d of %d uploaded",
                     ctx->max_smear_table, ctx->n_track_tables);
  return PP_OK;
}

// Grid and safety field go to shared memory when two CTAs of the configured
// size still fit on an SM; otherwise both are read from global memory.
bool use_smem_grid(const pp_ctx* ctx) {
  if (ctx->tuning.grid_in_global) return false;
  return pp::propagate_smem_bytes(ctx->grid.blob_bytes, ctx->sgrid.bytes, true,
                                  ctx->tuning.block_threads, nullptr, nullptr) <=
         pp::smem_budget(ctx->tuning.block_threads);
}

LaunchArgs make_args(const pp_ctx* ctx, long long seed, int n_steps, pp_hit_record* hits,
                     long long capacity, pp_counters* ctr) {
  LaunchArgs a{};
  a.sources = ctx->d_sources;
  a.chunk_prefix = ctx->d_prefix;
  a.src_photons = ctx->d_src_photons;
  a.total_chunks = ctx->total_chunks;
  a.n_src = ctx->n_src;
  a.chunk_photons = ctx->chunk_photons;
  a.blob = ctx->d_blob;
  a.grid = ctx->grid;
  a.safety = ctx->d_safety;
  a.shapes = ctx->n_shapes > 0 ? ctx->d_shapes : nullptr;
  a.n_shapes = ctx->n_shapes;
  if (ctx->n_shapes == 0 && ctx->tuning.target_loop && !ctx->h_targets.empty()) {
    a.shapes = ctx->d_loop_spheres;
    a.n_shapes = (int)ctx->h_targets.size();
  }
  a.sgrid = ctx->sgrid;
  a.medium = ctx->d_medium;
  a.n_medium = ctx->n_medium;
  a.med_wl_min = ctx->med_wl_min;
  a.med_inv_step = ctx->med_inv_step;
  a.phase = ctx->phase;
  a.spectrum = ctx->n_spectrum > 0 ? ctx->d_spectrum : nullptr;
  a.n_spectrum = ctx->n_spectrum;
  a.mono_wavelength = ctx->mono;
  a.track = ctx->d_track;
  a.n_track = ctx->n_track;
  a.set_seed((uint64_t)seed);
  a.n_steps = n_steps;
  a.hits = hits;
  a.capacity = capacity > 0 ? (unsigned long long)capacity : 0ull;
  a.counters = ctr;
  a.wait_limit_ns = 2000000000ull;
  return a;
}

int enqueue(pp_ctx* ctx, long long seed, int n_steps, pp_hit_record* d_hits, long long capacity,
            pp_counters* d_ctr, cudaStream_t stream) {
  PP_CUDA(cudaMemsetAsync(d_ctr, 0, sizeof(pp_counters), stream), "zero counters");
  if (ctx->total_chunks == 0) return PP_OK;
  const LaunchArgs a = make_args(ctx, seed, n_steps, d_hits, capacity, d_ctr);
  int grid = 0;
  cudaError_t e = pp::launch_propagate(a, ctx->tuning.block_threads, ctx->tuning.ctas_per_sm,
                                       ctx->tuning.precise_math != 0, use_smem_grid(ctx),
                                       ctx->num_sms, stream, &grid);
  if (e != cudaSuccess) return cuda_error(e, "launch propagate kernel");
  return PP_OK;
}

int validate_launch(pp_ctx* ctx, int n_steps, const void* d_hits, long long capacity,
                    const void* d_ctr) {
  if (!ctx) return set_error(PP_ERR_INVALID, "null context");
  if (n_steps < 1 || n_steps > 65535)
    return set_error(PP_ERR_INVALID, "n_steps must be in [1, 65535] (got %d)", n_steps);
  if (!d_ctr) return set_error(PP_ERR_INVALID, "null counters pointer");
  if (capacity < 0) return set_error(PP_ERR_INVALID, "negative capacity");
  if (capacity > 0 && !d_hits) return set_error(PP_ERR_INVALID, "null hit buffer");
  if (((uintptr_t)d_hits & 15u) != 0) return set_error(PP_ERR_INVALID, "hit buffer not 16-byte aligned");
  return check_ready(ctx);
}

int fetch_hits(pp_ctx* ctx, const pp_hits* out, long long n);

// Block until the context's launches on callers' streams have finished.
void wait_launches(pp_ctx* ctx) {
  if (ctx && ctx->inflight) cudaEventSynchronize(ctx->inflight);
}
void mark_launch(pp_ctx* ctx, cudaStream_t s) {
  if (ctx->inflight) cudaEventRecord(ctx->inflight, s);
}

}  // namespace

extern "C" {

PP_API int pp_version(void) { return PP_ABI_VERSION; }

PP_API int pp_last_error(char* buf, int32_t len) {
  const int n = (int)g_last_error.size();
  if (buf && len > 0) {
    const int m = std::min(n, len - 1);
    memcpy(buf, g_last_error.data(), m);
    buf[m] = '\0';
  }
  return n;
}

PP_API int pp_create(pp_ctx** out, int32_t device) {
  if (!out) return set_error(PP_ERR_INVALID, "null output pointer");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(PP_ERR_NO_DEVICE, "no CUDA device available (%s)",
                     e != cudaSuccess ? cudaGetErrorString(e) : "device count is 0");
  }
  if (device < 0 || device >= count)
    return set_error(PP_ERR_INVALID, "device %d out of range [0, %d)", device, count);
  DeviceScope ds(device);
  pp_ctx* ctx = new pp_ctx();
  ctx->device = device;
  e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->inflight, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_ctr, sizeof(pp_counters));
  if (e != cudaSuccess) {
    int rc = cuda_error(e, "pp_create");
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return rc;
  }
  *out = ctx;
  return PP_OK;
}

PP_API int pp_destroy(pp_ctx* ctx) {
  if (!ctx) return PP_OK;
  DeviceScope ds(ctx->device);
  wait_launches(ctx);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->gexec) cudaGraphExecDestroy(ctx->gexec);
  cudaFree(ctx->d_medium);
  cudaFree(ctx->d_es_table);
  cudaFree(ctx->d_spectrum);
  cudaFree(ctx->d_track);
  cudaFree(ctx->d_targets);
  cudaFree(ctx->d_shapes);
  cudaFree(ctx->d_loop_spheres);
  cudaFree(ctx->d_blob);
  cudaFree(ctx->d_safety);
  cudaFree(ctx->d_sources);
  cudaFree(ctx->d_prefix);
  cudaFree(ctx->d_src_photons);
  cudaFree(ctx->d_hits);
  cudaFree(ctx->d_ctr);
  if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->inflight) cudaEventDestroy(ctx->inflight);
  delete ctx;
  return PP_OK;
}

PP_API int pp_set_medium(pp_ctx* ctx, const pp_medium* m) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || !m) return set_error(PP_ERR_INVALID, "null argument");
  if (m->n_knots < 2 || !(m->wl_step > 0.0f) || !std::isfinite(m->wl_min))
    return set_error(PP_ERR_INVALID, "medium grid needs n_knots >= 2 and wl_step > 0");
  if (!m->scattering_length || !m->group_velocity || !m->absorption_length ||
      !m->phase_refractive_index)
    return set_error(PP_ERR_INVALID, "medium table pointer is null");
  pp::PhaseDev phase{};
  if (const char* why = pp::make_phase(m, &phase)) return set_error(PP_ERR_INVALID, "%s", why);
  std::vector<float4> t(m->n_knots);
  for (int i = 0; i < m->n_knots; ++i) {
    const float s = m->scattering_length[i], v = m->group_velocity[i];
    const float ab = m->absorption_length[i], n = m->phase_refractive_index[i];
    if (!(s > 0.0f) || !(v > 0.0f) || !(ab > 0.0f) || !(n > 0.0f) || !std::isfinite(s) ||
        !std::isfinite(v) || !std::isfinite(n))
      return set_error(PP_ERR_INVALID, "medium table entry %d is not positive and finite", i);
    t[i] = make_float4(s, v, ab, n);
  }
  DeviceScope ds(ctx->device);
  cudaFree(ctx->d_medium);
  ctx->d_medium = nullptr;
  PP_CUDA(cudaMalloc(&ctx->d_medium, sizeof(float4) * t.size()), "cudaMalloc(medium)");
  PP_CUDA(cudaMemcpy(ctx->d_medium, t.data(), sizeof(float4) * t.size(), cudaMemcpyHostToDevice),
          "upload medium");
  ctx->n_medium = m->n_knots;
  ctx->med_wl_min = m->wl_min;
  ctx->med_inv_step = 1.0f / m->wl_step;
  cudaFree(ctx->d_es_table);
  ctx->d_es_table = nullptr;
  if (phase.kind == PP_PHASE_HG_ES && m->hg_weight < 1.0f) {
    std::vector<float2> es(pp::kEsTable);
    pp::make_es_table(phase.es_b, es.data());
    PP_CUDA(cudaMalloc(&ctx->d_es_table, sizeof(float2) * es.size()), "cudaMalloc(ES table)");
    PP_CUDA(cudaMemcpy(ctx->d_es_table, es.data(), sizeof(float2) * es.size(),
                       cudaMemcpyHostToDevice),
            "upload ES table");
  }
  phase.es_table = ctx->d_es_table;
  ctx->phase = phase;
  ctx->has_medium = true;
  ctx->version++;
  return PP_OK;
}

PP_API int pp_set_spectrum(pp_ctx* ctx, const float* knots, int32_t n) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || !knots || n < 1) return set_error(PP_ERR_INVALID, "spectrum needs n >= 1 knots");
  for (int i = 0; i < n; ++i)
    if (!(knots[i] > 0.0f) || !std::isfinite(knots[i]))
      return set_error(PP_ERR_INVALID, "spectrum knot %d is not a positive wavelength", i);
  DeviceScope ds(ctx->device);
  cudaFree(ctx->d_spectrum);
  ctx->d_spectrum = nullptr;
  PP_CUDA(cudaMalloc(&ctx->d_spectrum, sizeof(float) * n), "cudaMalloc(spectrum)");
  PP_CUDA(cudaMemcpy(ctx->d_spectrum, knots, sizeof(float) * n, cudaMemcpyHostToDevice),
          "upload spectrum");
  ctx->n_spectrum = n;
  ctx->has_spectrum = true;
  ctx->version++;
  return PP_OK;
}

PP_API int pp_set_monochromatic(pp_ctx* ctx, float wavelength) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || !(wavelength > 0.0f) || !std::isfinite(wavelength))
    return set_error(PP_ERR_INVALID, "monochromatic wavelength must be positive");
  DeviceScope ds(ctx->device);
  cudaFree(ctx->d_spectrum);
  ctx->d_spectrum = nullptr;
  ctx->n_spectrum = 0;
  ctx->mono = wavelength;
  ctx->has_spectrum = true;
  ctx->version++;
  return PP_OK;
}

PP_API int pp_set_track_smear_tables(pp_ctx* ctx, const float* q, int32_t n, int32_t n_tables) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || !q || n < 2) return set_error(PP_ERR_INVALID, "track table needs n >= 2 knots");
  if (n_tables < 1 || (long long)n * n_tables > (1ll << 26))
    return set_error(PP_ERR_INVALID, "track tables: need 1 <= n_tables and n * n_tables <= 2^26");
  const long long total = (long long)n * n_tables;
  for (long long i = 0; i < total; ++i)
    if (!(q[i] >= -1.0f && q[i] <= 1.0f))
      return set_error(PP_ERR_INVALID, "track quantile %lld outside [-1, 1]", i);
  DeviceScope ds(ctx->device);
  cudaFree(ctx->d_track);
  ctx->d_track = nullptr;
  ctx->n_track = 0;
  ctx->n_track_tables = 0;
  PP_CUDA(cudaMalloc(&ctx->d_track, sizeof(float) * total), "cudaMalloc(track)");
  PP_CUDA(cudaMemcpy(ctx->d_track, q, sizeof(float) * total, cudaMemcpyHostToDevice),
          "upload track");
  ctx->n_track = n;
  ctx->n_track_tables = n_tables;
  ctx->version++;
  return PP_OK;
}

PP_API int pp_set_track_smear(pp_ctx* ctx, const float* q, int32_t n) {
  return pp_set_track_smear_tables(ctx, q, n, 1);
}

PP_API int pp_set_targets(pp_ctx* ctx, const pp_sphere* t, int32_t n, float cell_size) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || n < 0 || (n > 0 && !t)) return set_error(PP_ERR_INVALID, "bad target list");
  if (n > 65535) return set_error(PP_ERR_INVALID, "at most 65535 targets are supported");
  for (int i = 0; i < n; ++i) {
    if (!(t[i].radius > 0.0f) || !std::isfinite(t[i].radius) || !std::isfinite(t[i].position[0]) ||
        !std::isfinite(t[i].position[1]) || !std::isfinite(t[i].position[2]))
      return set_error(PP_ERR_INVALID, "target %d has a non-finite position or radius <= 0", i);
  }
  DeviceScope ds(ctx->device);
  cudaFree(ctx->d_shapes);
  ctx->d_shapes = nullptr;
  ctx->n_shapes = 0;
  ctx->h_targets.assign(t, t + n);
  cudaFree(ctx->d_targets);
  ctx->d_targets = nullptr;
  cudaFree(ctx->d_loop_spheres);
  ctx->d_loop_spheres = nullptr;
  if (n > 0) {
    PP_CUDA(cudaMalloc(&ctx->d_targets, sizeof(pp_sphere) * n), "cudaMalloc(targets)");
    PP_CUDA(cudaMemcpy(ctx->d_targets, t, sizeof(pp_sphere) * n, cudaMemcpyHostToDevice),
            "upload targets");
    // the same spheres as shape records, for the unculled loop (target_loop)
    std::vector<float4> h(2 * (size_t)n);
    int kind = PP_TARGET_SPHERE;
    float kf;
    memcpy(&kf, &kind, sizeof(kf));
    for (int i = 0; i < n; ++i) {
      h[2 * i] = make_float4(t[i].position[0], t[i].position[1], t[i].position[2],
                             t[i].radius * t[i].radius);
      h[2 * i + 1] = make_float4(0.0f, kf, 0.0f, 0.0f);
    }
    PP_CUDA(cudaMalloc(&ctx->d_loop_spheres, sizeof(float4) * h.size()), "cudaMalloc(loop targets)");
    PP_CUDA(cudaMemcpy(ctx->d_loop_spheres, h.data(), sizeof(float4) * h.size(),
                       cudaMemcpyHostToDevice),
            "upload loop targets");
  }
  const float h = cell_size > 0.0f ? cell_size : ctx->tuning.cell_size;
  int rc = rebuild_grid(ctx, h);
  if (rc != PP_OK) {
    ctx->has_targets = false;
    return rc;
  }
  ctx->has_targets = true;
  return PP_OK;
}

PP_API int pp_set_shaped_targets(pp_ctx* ctx, const pp_target* t, int32_t n) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || n < 0 || (n > 0 && !t)) return set_error(PP_ERR_INVALID, "bad target list");
  if (n > 65535) return set_error(PP_ERR_INVALID, "at most 65535 targets are supported");
  // DetectorLines: groups of one line record and its N modules
  const bool lines = n > 0 && t[0].kind == PP_TARGET_LINE;
  const int per_line = lines ? t[0].reserved : 0;
  if (lines) {
    if (per_line < 1 || per_line >= n || n % (per_line + 1) != 0)
      return set_error(PP_ERR_INVALID, "detector lines: %d records are not groups of 1 + %d", n,
                       per_line);
    const long long n_lines = n / (per_line + 1);
    if ((long long)per_line * (n_lines + 1) > 65535)
      return set_error(PP_ERR_INVALID, "detector lines: module index N * (L + 1) exceeds 65535");
  }
  bool spheres_only = !lines;
  for (int i = 0; i < n; ++i) {
    const pp_target& x = t[i];
    if (!std::isfinite(x.position[0]) || !std::isfinite(x.position[1]) ||
        !std::isfinite(x.position[2]))
      return set_error(PP_ERR_INVALID, "target %d has a non-finite position", i);
    const bool line_slot = lines && i % (per_line + 1) == 0;
    if (line_slot != (x.kind == PP_TARGET_LINE))
      return set_error(PP_ERR_INVALID, "target %d: line records must head each group of %d modules",
                       i, per_line);
    if (x.kind == PP_TARGET_LINE) {
      if (x.reserved != per_line)
        return set_error(PP_ERR_INVALID, "target %d: every line must hold %d modules", i, per_line);
      if (!(x.radius > 0.0f) || !std::isfinite(x.radius))
        return set_error(PP_ERR_INVALID, "target %d: line radius must be > 0", i);
    } else if (x.kind == PP_TARGET_SPHERE || x.kind == PP_TARGET_DISC) {
      if (!(x.radius > 0.0f) || !std::isfinite(x.radius))
        return set_error(PP_ERR_INVALID, "target %d: radius must be > 0", i);
    } else if (x.kind == PP_TARGET_RECTANGLE) {
      if (!(x.length_x > 0.0f) || !(x.length_y > 0.0f) || !std::isfinite(x.length_x) ||
          !std::isfinite(x.length_y))
        return set_error(PP_ERR_INVALID, "target %d: rectangle lengths must be > 0", i);
    } else {
      return set_error(PP_ERR_INVALID, "target %d: unknown kind %d", i, x.kind);
    }
    spheres_only = spheres_only && x.kind == PP_TARGET_SPHERE;
  }
  if (spheres_only) {
    std::vector<pp_sphere> sp(n);
    for (int i = 0; i < n; ++i) {
      for (int k = 0; k < 3; ++k) sp[i].position[k] = t[i].position[k];
      sp[i].radius = t[i].radius;
    }
    return pp_set_targets(ctx, n ? sp.data() : nullptr, n, 0.0f);
  }
  // no culling grid: an empty sphere list, then the shapes
  int rc = pp_set_targets(ctx, nullptr, 0, 0.0f);
  if (rc != PP_OK) return rc;
  DeviceScope ds(ctx->device);
  std::vector<float4> h(2 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const pp_target& x = t[i];
    const bool rect = x.kind == PP_TARGET_RECTANGLE;
    const bool line = x.kind == PP_TARGET_LINE;
    const float p0 = rect ? 0.5f * x.length_x : x.radius * x.radius;
    float p1 = rect ? 0.5f * x.length_y : 0.0f;
    if (line) memcpy(&p1, &x.reserved, sizeof(p1));  // modules that follow
    int kind = x.kind;
    float kf;
    memcpy(&kf, &kind, sizeof(kf));
    h[2 * i] = make_float4(x.position[0], x.position[1], line ? 0.0f : x.position[2], p0);
    h[2 * i + 1] = make_float4(p1, kf, 0.0f, 0.0f);
  }
  PP_CUDA(cudaMalloc(&ctx->d_shapes, sizeof(float4) * h.size()), "cudaMalloc(shaped targets)");
  PP_CUDA(cudaMemcpy(ctx->d_shapes, h.data(), sizeof(float4) * h.size(), cudaMemcpyHostToDevice),
          "upload shaped targets");
  ctx->n_shapes = n;
  ctx->version++;
  return PP_OK;
}

PP_API int pp_set_sources(pp_ctx* ctx, const pp_source* s, int32_t n, float photon_scaling) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || n < 0 || (n > 0 && !s)) return set_error(PP_ERR_INVALID, "bad source list");
  if (!(photon_scaling >= 0.0f) || !std::isfinite(photon_scaling))
    return set_error(PP_ERR_INVALID, "photon_scaling must be finite and >= 0");
  bool needs_track = false;
  int max_table = 0;
  for (int i = 0; i < n; ++i) {
    const pp_source& x = s[i];
    if (x.kind < 0 || x.kind >= PP_SRC_KIND_COUNT)
      return set_error(PP_ERR_INVALID, "source %d has unknown kind %d", i, x.kind);
    if (x.photons < 0) return set_error(PP_ERR_INVALID, "source %d has negative photons", i);
    if (x.kind == PP_SRC_EXTENDED_CHERENKOV || x.kind == PP_SRC_EXTENDED_CHERENKOV_NOSMEAR) {
      if (!(x.long_a > 0.0f) || !(x.long_b > 0.0f) || !(x.long_lrad >= 0.0f))
        return set_error(PP_ERR_INVALID, "source %d: longitudinal parameters must be positive", i);
    }
    if (kind_uses_track(x.kind)) {
      if (x.smear_table < 0)
        return set_error(PP_ERR_INVALID, "source %d: negative track-smear table", i);
      needs_track = true;
      max_table = std::max(max_table, (int)x.smear_table);
    }
  }
  DeviceScope ds(ctx->device);
  ctx->h_sources.assign(s, s + n);
  ctx->scaling = photon_scaling;
  ctx->needs_track = needs_track;
  ctx->max_smear_table = max_table;
  int rc = build_queue(ctx);
  ctx->has_sources = rc == PP_OK;
  return rc;
}

PP_API int pp_set_tuning(pp_ctx* ctx, const pp_tuning* t) {
  wait_launches(ctx);  // inputs of launches in flight are about to change
  if (!ctx || !t) return set_error(PP_ERR_INVALID, "null argument");
  if (t->block_threads < 64 || t->block_threads > 1024 || (t->block_threads % 32) != 0)
    return set_error(PP_ERR_INVALID, "block_threads must be a multiple of 32 in [64, 1024]");
  if (t->safety_cell < 0.0f) return set_error(PP_ERR_INVALID, "safety_cell must be >= 0");
  if (t->photons_per_thread < 1 || t->photons_per_thread > 4096)
    return set_error(PP_ERR_INVALID, "photons_per_thread must be in [1, 4096]");
  if (t->ctas_per_sm < 0) return set_error(PP_ERR_INVALID, "ctas_per_sm must be >= 0");
  if (t->target_loop != 0 && t->target_loop != 1)
    return set_error(PP_ERR_INVALID, "target_loop must be 0 or 1");
  DeviceScope ds(ctx->device);
  const bool ppt_changed = t->photons_per_thread != ctx->tuning.photons_per_thread;
  const bool cell_changed =
      t->cell_size != ctx->tuning.cell_size || t->safety_cell != ctx->tuning.safety_cell;
  ctx->tuning = *t;
  ctx->version++;
  if (ppt_changed && ctx->has_sources) {
    int rc = build_queue(ctx);
    if (rc != PP_OK) return rc;
  }
  if (cell_changed && ctx->has_targets) {
    int rc = rebuild_grid(ctx, t->cell_size);
    if (rc != PP_OK) return rc;
  }
  return PP_OK;
}

PP_API int pp_get_tuning(const pp_ctx* ctx, pp_tuning* t) {
  if (!ctx || !t) return set_error(PP_ERR_INVALID, "null argument");
  *t = ctx->tuning;
  return PP_OK;
}

PP_API int pp_total_photons(const pp_ctx* ctx, int64_t* total) {
  if (!ctx || !total) return set_error(PP_ERR_INVALID, "null argument");
  *total = ctx->total_photons;
  return PP_OK;
}

PP_API int pp_launch(pp_ctx* ctx, int64_t seed, int32_t n_steps, pp_hit_record* d_hits,
                     int64_t capacity, pp_counters* d_counters, void* stream) {
  int rc = validate_launch(ctx, n_steps, d_hits, capacity, d_counters);
  if (rc != PP_OK) return rc;
  DeviceScope ds(ctx->device);
  rc = enqueue(ctx, seed, n_steps, d_hits, capacity, d_counters, (cudaStream_t)stream);
  if (rc == PP_OK) mark_launch(ctx, (cudaStream_t)stream);
  return rc;
}

PP_API int pp_debug_staging_timeout(pp_ctx* ctx, int64_t wait_ns) {
  if (!ctx) return set_error(PP_ERR_INVALID, "null context");
  int rc = check_ready(ctx);
  if (rc != PP_OK) return rc;
  if (wait_ns < 1000 || wait_ns > 2000000000)
    return set_error(PP_ERR_INVALID, "wait_ns must be in [1e3, 2e9]");
  if (ctx->total_chunks == 0 || ctx->h_targets.empty() || ctx->n_shapes > 0 ||
      ctx->tuning.target_loop || !use_smem_grid(ctx))
    return set_error(PP_ERR_INVALID,
                     "the staging wait needs sources, a sphere list and tables in shared memory");
  DeviceScope ds(ctx->device);
  pp_counters* d_ctr = nullptr;
  PP_CUDA(cudaMalloc(&d_ctr, sizeof(pp_counters)), "cudaMalloc(counters)");
  LaunchArgs a = make_args(ctx, 1, 1, nullptr, 0, d_ctr);
  a.wait_limit_ns = (unsigned long long)wait_ns;
  a.skip_staging_copies = 1;
  pp_counters c{};
  cudaError_t e = cudaMemsetAsync(d_ctr, 0, sizeof(pp_counters), ctx->stream);
  if (e == cudaSuccess)
    e = pp::launch_propagate(a, ctx->tuning.block_threads, ctx->tuning.ctas_per_sm,
                             ctx->tuning.precise_math != 0, true, ctx->num_sms, ctx->stream,
                             nullptr);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&c, d_ctr, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  cudaFree(d_ctr);
  if (e != cudaSuccess) return cuda_error(e, "staging-timeout diagnostic");
  if (c.err_flags & PP_FLAG_TIMEOUT)
    return set_error(PP_ERR_TIMEOUT, "a bounded device wait (TMA staging) timed out");
  return PP_OK;
}

PP_API int pp_launch_histogram(pp_ctx* ctx, int64_t seed, int32_t n_steps, const float* d_tgeo,
                               float* d_hist, int32_t n_bins, float t_offset, float log_lo,
                               float log_hi, pp_counters* d_counters, void* stream) {
  int rc = validate_launch(ctx, n_steps, nullptr, 0, d_counters);
  if (rc != PP_OK) return rc;
  if (!d_tgeo || !d_hist || n_bins < 1 || !(log_hi > log_lo))
    return set_error(PP_ERR_INVALID, "histogram needs tgeo, hist, n_bins >= 1, log_hi > log_lo");
  DeviceScope ds(ctx->device);
  cudaStream_t s = (cudaStream_t)stream;
  PP_CUDA(cudaMemsetAsync(d_counters, 0, sizeof(pp_counters), s), "zero counters");
  PP_CUDA(cudaMemsetAsync(d_hist, 0, sizeof(float) * (size_t)ctx->n_src * (n_bins + 1), s),
          "zero histograms");
  if (ctx->total_chunks == 0) return PP_OK;
  LaunchArgs a = make_args(ctx, seed, n_steps, nullptr, 0, d_counters);
  a.hist = d_hist;
  a.hist_tgeo = d_tgeo;
  a.hist_bins = n_bins;
  a.hist_t_offset = t_offset;
  a.hist_log_lo = log_lo;
  a.hist_inv_log_width = (float)n_bins / (log_hi - log_lo);
  cudaError_t e = pp::launch_propagate(a, ctx->tuning.block_threads, ctx->tuning.ctas_per_sm,
                                       ctx->tuning.precise_math != 0, use_smem_grid(ctx),
                                       ctx->num_sms, s, nullptr);
  if (e != cudaSuccess) return cuda_error(e, "launch propagate kernel (histogram)");
  mark_launch(ctx, s);
  return PP_OK;
}

PP_API int pp_launch_graph(pp_ctx* ctx, int64_t seed, int32_t n_steps, pp_hit_record* d_hits,
                           int64_t capacity, pp_counters* d_counters, void* stream) {
  int rc = validate_launch(ctx, n_steps, d_hits, capacity, d_counters);
  if (rc != PP_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  if (s == nullptr || s == cudaStreamLegacy || s == cudaStreamPerThread)
    return set_error(PP_ERR_INVALID, "pp_launch_graph needs a created (non-default) stream");
  DeviceScope ds(ctx->device);
  GraphKey key;
  key.seed = seed;
  key.n_steps = n_steps;
  key.hits = d_hits;
  key.capacity = capacity;
  key.counters = d_counters;
  key.stream = s;
  key.version = ctx->version;
  if (!ctx->gexec || !(ctx->gkey == key)) {
    if (ctx->gexec) {
      cudaGraphExecDestroy(ctx->gexec);
      ctx->gexec = nullptr;
    }
    PP_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
    int erc = enqueue(ctx, seed, n_steps, d_hits, capacity, d_counters, s);
    cudaGraph_t graph = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (erc != PP_OK) {
      if (graph) cudaGraphDestroy(graph);
      return erc;
    }
    if (ce != cudaSuccess) return cuda_error(ce, "end capture");
    ce = cudaGraphInstantiate(&ctx->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      ctx->gexec = nullptr;
      return cuda_error(ce, "instantiate graph");
    }
    ctx->gkey = key;
  }
  PP_CUDA(cudaGraphLaunch(ctx->gexec, s), "graph launch");
  mark_launch(ctx, s);
  return PP_OK;
}

PP_API int pp_hits_to_columns(const pp_hit_record* d_records, int64_t n, const pp_hits* d_out,
                              void* stream) {
  if (n < 0 || !d_out || (n > 0 && !d_records)) return set_error(PP_ERR_INVALID, "bad arguments");
  cudaError_t e = pp::launch_hits_to_columns(d_records, n, *d_out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_error(e, "hits_to_columns");
  return PP_OK;
}

PP_API int pp_propagate(pp_ctx* ctx, const pp_source* sources, int32_t n_src, int64_t seed,
                        int32_t n_steps, float photon_scaling, const pp_hits* out,
                        int64_t capacity, int64_t* n_hits, int64_t* n_ph_sim) {
  if (!ctx || !n_hits || !n_ph_sim) return set_error(PP_ERR_INVALID, "null argument");
  if (capacity < 0) return set_error(PP_ERR_INVALID, "negative capacity");
  if (n_steps < 1) return set_error(PP_ERR_INVALID, "n_steps must be >= 1");
  *n_hits = 0;
  *n_ph_sim = 0;
  ctx->last_hits = 0;
  DeviceScope ds(ctx->device);
  int rc = pp_set_sources(ctx, sources, n_src, photon_scaling);
  if (rc != PP_OK) return rc;
  rc = check_ready(ctx);
  if (rc != PP_OK) return rc;
  // A photon hits at most once: the device buffer never needs more rows than
  // there are photons.
  const long long dev_cap = std::max<long long>(1, std::min<long long>(capacity, ctx->total_photons));
  if (dev_cap > ctx->d_hits_cap) {
    cudaFree(ctx->d_hits);
    ctx->d_hits = nullptr;
    ctx->d_hits_cap = 0;
    PP_CUDA(cudaMalloc(&ctx->d_hits, sizeof(pp_hit_record) * dev_cap), "cudaMalloc(hit buffer)");
    ctx->d_hits_cap = dev_cap;
  }
  rc = enqueue(ctx, seed, n_steps, ctx->d_hits, std::min<long long>(capacity, dev_cap), ctx->d_ctr,
               ctx->stream);
  if (rc != PP_OK) return rc;
  pp_counters c{};
  PP_CUDA(cudaMemcpyAsync(&c, ctx->d_ctr, sizeof(c), cudaMemcpyDeviceToHost, ctx->stream),
          "read counters");
  PP_CUDA(cudaStreamSynchronize(ctx->stream), "propagate");
  *n_hits = (int64_t)c.n_hits;
  *n_ph_sim = (int64_t)c.n_ph_sim;
  if (c.err_flags & PP_FLAG_TIMEOUT)
    return set_error(PP_ERR_TIMEOUT, "a bounded device wait (TMA staging) timed out");
  if ((c.err_flags & PP_FLAG_OVERFLOW) || (long long)c.n_hits > capacity)
    return set_error(PP_ERR_OVERFLOW, "hit buffer overflow: %llu hits, capacity %lld",
                     (unsigned long long)c.n_hits, (long long)capacity);
  const long long n = (long long)c.n_hits;
  ctx->last_hits = n;
  if (n == 0 || !out) return PP_OK;
  return fetch_hits(ctx, out, n);
}

PP_API int pp_fetch_hits(pp_ctx* ctx, const pp_hits* out, int64_t n) {
  if (!ctx || !out || n < 0) return set_error(PP_ERR_INVALID, "bad arguments");
  if (n > ctx->last_hits)
    return set_error(PP_ERR_INVALID, "only %lld hits are held", (long long)ctx->last_hits);
  if (n == 0) return PP_OK;
  DeviceScope ds(ctx->device);
  return fetch_hits(ctx, out, n);
}

PP_API int pp_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(PP_ERR_NO_DEVICE, "no CUDA device available");
  }
  if (device < 0 || device >= count) return set_error(PP_ERR_INVALID, "bad device");
  DeviceScope ds(device);
  size_t f = 0, t = 0;
  PP_CUDA(cudaMemGetInfo(&f, &t), "cudaMemGetInfo");
  if (free_bytes) *free_bytes = (int64_t)f;
  if (total_bytes) *total_bytes = (int64_t)t;
  return PP_OK;
}

}  // extern "C"

namespace {

int fetch_hits(pp_ctx* ctx, const pp_hits* out, long long n) {
  const void* first = out->position ? (const void*)out->position
                      : out->time   ? (const void*)out->time
                      : out->module_index ? (const void*)out->module_index
                                          : (const void*)out->wavelength;
  if (first && is_device_pointer(first)) {
    cudaError_t e = pp::launch_hits_to_columns(ctx->d_hits, n, *out, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_error(e, "hits_to_columns");
    return PP_OK;
  }
  if (n > ctx->h_stage_cap) {
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    ctx->h_stage = nullptr;
    ctx->h_stage_cap = 0;
    PP_CUDA(cudaMallocHost(&ctx->h_stage, sizeof(pp_hit_record) * n), "cudaMallocHost(stage)");
    ctx->h_stage_cap = n;
  }
  PP_CUDA(cudaMemcpyAsync(ctx->h_stage, ctx->d_hits, sizeof(pp_hit_record) * n,
                          cudaMemcpyDeviceToHost, ctx->stream),
          "copy hits");
  PP_CUDA(cudaStreamSynchronize(ctx->stream), "copy hits");
  for (long long i = 0; i < n; ++i) {
    const pp_hit_record& h = ctx->h_stage[i];
    for (int a = 0; a < 3; ++a) {
      if (out->position) out->position[3 * i + a] = h.position[a];
      if (out->direction) out->direction[3 * i + a] = h.direction[a];
      if (out->initial_direction) out->initial_direction[3 * i + a] = h.initial_direction[a];
    }
    if (out->wavelength) out->wavelength[i] = h.wavelength;
    if (out->time) out->time[i] = h.time;
    if (out->dist_travelled) out->dist_travelled[i] = h.dist_travelled;
    if (out->abs_weight) out->abs_weight[i] = h.abs_weight;
    if (out->module_index) out->module_index[i] = h.module_index;
    if (out->n_steps) out->n_steps[i] = h.n_steps;
    if (out->source_index) out->source_index[i] = h.source_index;
    if (out->photon_index) out->photon_index[i] = h.photon_index;
  }
  return PP_OK;
}

}  // namespace

extern "C" {

PP_API int pp_autotune(pp_ctx* ctx, int64_t seed, int32_t n_steps, int64_t sample_photons,
                       pp_tuning* best_out, double* best_rate) {
  if (!ctx) return set_error(PP_ERR_INVALID, "null context");
  int rc = check_ready(ctx);
  if (rc != PP_OK) return rc;
  if (n_steps < 1) return set_error(PP_ERR_INVALID, "n_steps must be >= 1");
  if (ctx->total_photons <= 0) return set_error(PP_ERR_INVALID, "no photons to tune on");
  DeviceScope ds(ctx->device);
  const std::vector<pp_source> orig = ctx->h_sources;
  const float orig_scaling = ctx->scaling;
  const pp_tuning orig_tuning = ctx->tuning;

  // Sample: every source scaled by the same factor (at least one photon).
  const long long want = sample_photons > 0 ? sample_photons : 4000000;
  const double f = std::min(1.0, (double)want / (double)ctx->total_photons);
  std::vector<pp_source> sample = orig;
  for (auto& s : sample) {
    const long long n = source_photons(s.photons, orig_scaling);
    s.photons = n > 0 ? std::max<long long>(1, (long long)std::llround(n * f)) : 0;
  }
  ctx->h_sources = sample;
  ctx->scaling = 1.0f;

  pp_hit_record* d_hits = nullptr;
  pp_counters* d_ctr = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  long long cap = 0;
  for (const auto& s : sample) cap += s.photons;
  cap = std::max<long long>(cap, 1);
  auto finish = [&](int code) {
    cudaFree(d_hits);
    cudaFree(d_ctr);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    ctx->h_sources = orig;
    ctx->scaling = orig_scaling;
    return code;
  };
  if (cudaMalloc(&d_hits, sizeof(pp_hit_record) * cap) != cudaSuccess ||
      cudaMalloc(&d_ctr, sizeof(pp_counters)) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    ctx->tuning = orig_tuning;
    finish(0);
    build_queue(ctx);
    return set_error(PP_ERR_CUDA, "autotune: allocation failed");
  }

  auto time_config = [&](const pp_tuning& t, double* ms_out) -> int {
    ctx->tuning = t;
    int r = build_queue(ctx);
    if (r != PP_OK) return r;
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
      cudaEventRecord(e0, ctx->stream);
      r = enqueue(ctx, seed, n_steps, d_hits, cap, d_ctr, ctx->stream);
      if (r != PP_OK) return r;
      cudaEventRecord(e1, ctx->stream);
      cudaError_t ce = cudaEventSynchronize(e1);
      if (ce != cudaSuccess) return cuda_error(ce, "autotune launch");
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) best = std::min(best, ms);
    }
    *ms_out = best;
    return PP_OK;
  };

  // Stage 1: grid cell size, then stage 2: safety-field cell size, both at a
  // 1024-thread launch; stage 3: launch shape at the chosen sizes.
  const float auto_h = ctx->grid.cell[0];
  const float auto_s = ctx->sgrid.cell;
  pp_tuning best = orig_tuning;
  best.block_threads = 1024;
  double best_ms = 1e300;
  if (!ctx->h_targets.empty()) {
    const float cell_factors[] = {0.75f, 1.0f, 1.5f, 2.0f};
    float best_h = auto_h;
    for (float cf : cell_factors) {
      pp_tuning t = best;
      t.cell_size = auto_h * cf;
      ctx->tuning.safety_cell = auto_s;
      if (rebuild_grid(ctx, t.cell_size) != PP_OK) continue;
      double ms;
      if (time_config(t, &ms) != PP_OK) continue;
      if (ms < best_ms) {
        best_ms = ms;
        best_h = t.cell_size;
      }
    }
    best.cell_size = best_h;
    best_ms = 1e300;
    const float safety_factors[] = {1.0f, 0.8f, 0.6f};
    float best_s = auto_s;
    for (float sf : safety_factors) {
      pp_tuning t = best;
      t.safety_cell = auto_s * sf;
      ctx->tuning.safety_cell = t.safety_cell;
      if (rebuild_grid(ctx, best_h) != PP_OK) continue;
      double ms;
      if (time_config(t, &ms) != PP_OK) continue;
      if (ms < best_ms) {
        best_ms = ms;
        best_s = t.safety_cell;
      }
    }
    best.safety_cell = best_s;
    ctx->tuning.safety_cell = best_s;
    if (rebuild_grid(ctx, best_h) != PP_OK) {
      ctx->tuning = orig_tuning;
      finish(0);
      build_queue(ctx);
      return PP_ERR_INVALID;
    }
  }
  // launch shape: the first candidate (one 1024-thread CTA per SM) is kept
  // unless another is more than 1% faster on the sample (sample timings vary
  // by about that much)
  best_ms = 1e300;
  const int blocks[] = {1024, 512};
  const int ppts[] = {8, 2};
  for (int b : blocks) {
    for (int p : ppts) {
      pp_tuning t = best;
      t.block_threads = b;
      t.photons_per_thread = p;
      double ms;
      if (time_config(t, &ms) != PP_OK) continue;
      if (ms < 0.99 * best_ms) {
        best_ms = ms;
        best.block_threads = b;
        best.photons_per_thread = p;
      }
    }
  }
  finish(0);
  ctx->tuning = best;
  rc = build_queue(ctx);
  if (rc != PP_OK) return rc;
  if (best_out) *best_out = best;
  if (best_rate) *best_rate = best_ms < 1e300 ? (double)cap / (best_ms * 1e-3) : 0.0;
  return best_ms < 1e300 ? PP_OK : set_error(PP_ERR_CUDA, "autotune: no configuration ran");
}

PP_API int pp_debug_philox(const uint32_t* ctr, int32_t n, uint32_t key0, uint32_t key1,
                           uint32_t* out) {
  if (!ctr || !out || n < 0) return set_error(PP_ERR_INVALID, "bad arguments");
  if (n == 0) return PP_OK;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(PP_ERR_NO_DEVICE, "no CUDA device available");
  }
  uint32_t *dc = nullptr, *dout = nullptr;
  const size_t bytes = sizeof(uint32_t) * 4 * (size_t)n;
  cudaError_t e = cudaMalloc(&dc, bytes);
  if (e == cudaSuccess) e = cudaMalloc(&dout, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(dc, ctr, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = pp::launch_debug_philox(dc, n, key0, key1, dout, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
  cudaFree(dc);
  cudaFree(dout);
  if (e != cudaSuccess) return cuda_error(e, "pp_debug_philox");
  return PP_OK;
}

PP_API int pp_measure_fp32_peak(int32_t device, double* tflops) {
  if (!tflops) return set_error(PP_ERR_INVALID, "null argument");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return set_error(PP_ERR_NO_DEVICE, "no CUDA device available");
  }
  DeviceScope ds(device);
  int sms = 0;
  PP_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "attribute");
  const int blocks = sms * 8, threads = 256, iters = 4096;
  float* sink = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMalloc(&sink, sizeof(float) * blocks);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  float best = 1e30f;
  for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
    cudaEventRecord(a, s);
    e = pp::launch_fp32_peak(sink, blocks, threads, iters, s);
    cudaEventRecord(b, s);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float ms = 0.0f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, a, b);
    if (rep > 0) best = std::min(best, ms);
  }
  cudaFree(sink);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) return cuda_error(e, "pp_measure_fp32_peak");
  const double flops = (double)blocks * threads * iters * 16.0 * 8.0 * 2.0;
  *tflops = flops / (best * 1e-3) / 1e12;
  return PP_OK;
}

PP_API int pp_grid_info(const pp_ctx* ctx, int32_t dims[3], float cell[3], float origin[3],
                        int64_t* n_items, int64_t* blob_bytes) {
  if (!ctx) return set_error(PP_ERR_INVALID, "null context");
  for (int a = 0; a < 3; ++a) {
    if (dims) dims[a] = ctx->grid.dims[a];
    if (cell) cell[a] = ctx->grid.cell[a];
    if (origin) origin[a] = ctx->grid.lo[a];
  }
  if (n_items) *n_items = ctx->n_items;
  if (blob_bytes) *blob_bytes = ctx->grid.blob_bytes;
  return PP_OK;
}

}  // extern "C"
