// pp_internal.h -- structures shared by the host runtime and the device
// kernels of the photon-transport library (not part of the public ABI).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "pp_gb300.h"

namespace pp {

// Uniform culling grid over the targets.  The grid, its per-cell candidate
// lists and the sphere table live in one contiguous 16-byte aligned "blob"
// that each CTA stages into shared memory with one TMA bulk copy:
//   [cells  : uint32 x n_cells, (count << 20) | first_item]  padded to 16 B
//   [items  : uint16 x n_items, target indices]             padded to 16 B
//   [spheres: float4 x n_targets, (x, y, z, r^2)]
struct GridDev {
  float lo[3];        // origin of cell (0,0,0)
  float hi[3];        // lo + dims * cell
  float cell[3];      // cell edge per axis (m)
  float inv_cell[3];  // 1 / cell
  int dims[3];
  int n_cells;
  int n_targets;
  uint32_t off_items;    // byte offset of the item list in the blob
  uint32_t off_spheres;  // byte offset of the sphere table in the blob
  uint32_t blob_bytes;   // multiple of 16
};

// Safety field: a coarser-or-finer uniform grid over the same box whose cell
// value is a lower bound on the distance from the cell centre to the nearest
// (inflated) sphere surface, quantised down in kSafetyQuantum steps (uint8).
// A step segment lies inside the ball of radius L/2 about its midpoint m; if
// D(centre) - |m - centre| > L/2 (1-Lipschitz) no sphere can be hit.
struct SafetyDev {
  float lo[3];
  float hi[3];
  float cell;      // edge (m), cubic cells
  float inv_cell;
  int dims[3];
  int n_cells;
  uint32_t bytes;  // allocation, n_cells rounded up to 16 (padding bytes are 0)
  // Derived on the host (set_derived) so that the kernel's tests read them
  // as constant operands instead of converting dims or re-adding offsets.
  float fdims[3];  // dims as float
  float fmaxc[3];  // dims - 1 as float (largest cell coordinate)
  float lo_sc[3];  // lo * inv_cell
  float c_lo[3];   // centre of cell 0: lo + cell / 2
  float bc[3];     // centre of the field's box
  float he[3];     // half extents of the field's box
  void set_derived() {
    for (int a = 0; a < 3; ++a) {
      fdims[a] = (float)dims[a];
      fmaxc[a] = (float)(dims[a] - 1);
      lo_sc[a] = lo[a] * inv_cell;
      c_lo[a] = lo[a] + 0.5f * cell;
      bc[a] = 0.5f * (lo[a] + hi[a]);
      he[a] = 0.5f * (hi[a] - lo[a]);
    }
  }
};
constexpr float kSafetyQuantum = 0.5f;  // m per uint8 step (saturates at 127.5 m)

// Per-warp shared-memory state of the propagation kernel: the queue of
// deferred step segments and, per lane, the earliest hit found so far.
// Entries [0, checked) of the queue have been clipped by the safety field and
// wait for the grid walk over [t0, t1]; entries from `checked` on wait to be
// clipped (at most 32 of them at a time).
constexpr int kQueueCap = 64;
constexpr int kMaxBlockThreads = 1024;
struct WarpQueue {
  float px[kQueueCap], py[kQueueCap], pz[kQueueCap];
  float dx[kQueueCap], dy[kQueueCap], dz[kQueueCap];
  float len[kQueueCap];
  float dist0[kQueueCap];     // compensated path length at the segment start
  uint32_t meta[kQueueCap];   // owner lane | step << 8
  float t0[kQueueCap];        // part of the segment the grid walk must cover
  float t1[kQueueCap];
};
struct WarpBest {
  uint32_t key[32];           // step << 16 | target index; ~0 = none
  float hx[32], hy[32], hz[32];
  float ox[32], oy[32], oz[32];
  float dist[32];
};

constexpr uint32_t kCellStartBits = 20;                    // first item index
constexpr uint32_t kCellStartMask = (1u << kCellStartBits) - 1u;
constexpr uint32_t kCellMaxCount = (1u << (32 - kCellStartBits)) - 1u;
constexpr float kGridMargin = 0.01f;                       // m, AABB inflation

// Phase-function constants derived once per medium.
struct PhaseDev {
  float hg_weight;  // P(Henyey-Greenstein)
  float hg_g;
  float hg_1mg2;    // 1 - g^2
  float hg_1pg2;    // 1 + g^2
  float hg_inv2g;   // 1 / (2 g)
  float es_k1;      // (b + 3) / b
  float es_k2;      // 1 / b^3
  float es_b;       // Einstein-Smoluchowski b
  int kind;         // PP_PHASE_*
  float sl_exp;     // simplified Liu: (1 - g) / (1 + g)
  // Einstein-Smoluchowski inverse CDF for the fast kernel: kEsTable intervals
  // of eta on [0, 1], entry i = {q(i / N), q((i + 1) / N) - q(i / N)} (set by
  // pp_set_medium; null: the Cardano formula)
  const float2* es_table;
};

// Intervals of the tabulated Einstein-Smoluchowski inverse CDF.  q(eta) is
// smooth on [0, 1] (its derivative is 1 / pdf, and pdf ~ 1 + b cos^2 is
// bounded away from 0), so linear interpolation on 1024 intervals is exact to
// ~1e-7, below the SFU cube roots of the formula it replaces.
constexpr int kEsTable = 1024;

// The table of PhaseDev::es_table for parameter b, in double and rounded once:
// q = cbrt(Q + D) + cbrt(Q - D), Q = (b + 3)(eta - 1/2) / b, D = sqrt(Q^2 + 1/b^3)
// (the Cardano root of the ES CDF's cubic, as the replay kernel evaluates it).
inline void make_es_table(float b, float2* out) {
  const double bb = b, k1 = (bb + 3.0) / bb, k2 = 1.0 / (bb * bb * bb);
  double prev = 0.0;
  for (int i = 0; i <= kEsTable; ++i) {
    const double q = k1 * ((double)i / kEsTable - 0.5);
    const double d = std::sqrt(q * q + k2);
    const double v = std::cbrt(q + d) + std::cbrt(q - d);
    if (i > 0) out[i - 1] = make_float2((float)prev, (float)(v - prev));
    prev = v;
  }
}

// The phase function of a medium, validated: nullptr on success, else the
// reason.  Shared by pp_set_medium and pp_propagate_static.
inline const char* make_phase(const pp_medium* m, PhaseDev* p) {
  if (m->phase_kind != PP_PHASE_HG_ES && m->phase_kind != PP_PHASE_HG_SL)
    return "phase_kind must be PP_PHASE_HG_ES or PP_PHASE_HG_SL";
  if (!(m->hg_weight >= 0.0f && m->hg_weight <= 1.0f)) return "hg_weight must be in [0, 1]";
  const float g = m->hg_g;
  if (m->hg_weight > 0.0f && !(std::fabs(g) >= 1e-3f && std::fabs(g) < 1.0f))
    return "hg_g must satisfy 1e-3 <= |g| < 1";
  if (m->phase_kind == PP_PHASE_HG_ES && m->hg_weight < 1.0f && !(m->es_b > 0.0f))
    return "es_b must be > 0 when the ES component is used";
  if (m->phase_kind == PP_PHASE_HG_SL && m->hg_weight < 1.0f && !(g > -1.0f && g < 1.0f))
    return "the simplified-Liu component needs -1 < g < 1";
  const float b = m->es_b > 0.0f ? m->es_b : 1.0f;
  p->hg_weight = m->hg_weight;
  p->hg_g = g;
  p->hg_1mg2 = 1.0f - g * g;
  p->hg_1pg2 = 1.0f + g * g;
  p->hg_inv2g = m->hg_weight > 0.0f ? 1.0f / (2.0f * g) : 0.0f;
  p->es_k1 = (b + 3.0f) / b;
  p->es_k2 = 1.0f / (b * b * b);
  p->es_b = b;
  p->kind = m->phase_kind;
  p->sl_exp = (1.0f - g) / (1.0f + g);
  return nullptr;
}

// Everything one launch of the propagation kernel needs (kernel parameter,
// passed as __grid_constant__).
struct LaunchArgs {
  const pp_source* sources;
  const unsigned long long* chunk_prefix;  // [n_src + 1] cumulative chunks
  const long long* src_photons;            // [n_src] photons after scaling
  unsigned long long total_chunks;
  int n_src;
  int chunk_photons;                       // 32 * photons_per_thread

  const unsigned char* blob;               // grid blob (global memory)
  GridDev grid;
  const unsigned char* safety;             // safety field (global memory)
  SafetyDev sgrid;
  // Shaped targets (no grid): 2 float4 per target, {x, y, z, p0} {p1, kind}:
  // sphere p0 = r^2; rectangle p0, p1 = half lengths; disc p0 = r^2.
  const float4* shapes;
  int n_shapes;

  const float4* medium;                    // {sca_len, v_group, abs_len, n}
  int n_medium;
  float med_wl_min;
  float med_inv_step;
  PhaseDev phase;

  const float* spectrum;                   // inverse CDF knots or nullptr
  int n_spectrum;
  float mono_wavelength;
  const float* track;                      // cos(theta) quantiles or nullptr
  int n_track;

  uint32_t key0, key1;                     // Philox key = seed
  uint32_t round_keys[20];                 // Philox round keys (set_seed)
  int n_steps;

  // key = seed; round r of Philox4x32-10 uses (key0 + r W0, key1 + r W1),
  // precomputed once per launch so that the per-step generator takes them as
  // kernel-parameter operands instead of recomputing them
  void set_seed(uint64_t seed) {
    key0 = (uint32_t)(seed & 0xffffffffu);
    key1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
      round_keys[2 * r] = key0 + (uint32_t)r * 0x9E3779B9u;
      round_keys[2 * r + 1] = key1 + (uint32_t)r * 0xBB67AE85u;
    }
  }

  pp_hit_record* hits;
  unsigned long long capacity;
  pp_counters* counters;
  unsigned long long wait_limit_ns;        // bound on the TMA staging wait
  int skip_staging_copies;                 // diagnostic: arm the barrier, copy nothing

  // Histogram mode (hist != nullptr): instead of hit records, every hit adds
  // its absorption weight to hist[s * (bins + 1)] (count) and to bin
  // 1 + b of log10(t - tgeo[s] + hist_t_offset) on [hist_log_lo, hist_log_hi).
  float* hist;
  const float* hist_tgeo;
  int hist_bins;
  float hist_t_offset;
  float hist_log_lo;
  float hist_inv_log_width;

  uint32_t safety_offset;                  // shared-memory offset of the staged field
  uint32_t state_offset;                   // shared-memory offset of the warp state
  int warps_per_block;
};

// Dynamic shared memory of one CTA: [grid blob | safety field] when staged,
// then the per-warp state.
inline size_t propagate_smem_bytes(uint32_t blob_bytes, uint32_t safety_bytes, bool smem_tables,
                                   int block_threads, uint32_t* safety_offset,
                                   uint32_t* state_offset) {
  const size_t blob = ((size_t)blob_bytes + 15) & ~(size_t)15;
  const size_t field = ((size_t)safety_bytes + 15) & ~(size_t)15;
  const size_t off = smem_tables ? blob + field : 0;
  if (safety_offset) *safety_offset = (uint32_t)blob;
  if (state_offset) *state_offset = (uint32_t)off;
  return off + (size_t)(block_threads / 32) * (sizeof(WarpQueue) + sizeof(WarpBest));
}
// Largest dynamic shared memory per CTA for which CTAs of block_threads
// still fill an SM with 1024 threads (the 64-register cap of the kernel): the
// SM's 228 KB less 1 KB reserved per CTA and the static barrier, at most the
// 227 KB one CTA may opt into.
inline size_t smem_budget(int block_threads) {
  const int ctas = block_threads >= 1024 ? 1 : 1024 / (block_threads > 0 ? block_threads : 1);
  const size_t b = (size_t)228 * 1024 / (size_t)ctas - 1024 - 64;
  return b < (size_t)227 * 1024 - 64 ? b : (size_t)227 * 1024 - 64;
}

// Host-side launch of the propagation kernel (pp_propagate.cu).
cudaError_t launch_propagate(const LaunchArgs& args, int block_threads, int ctas_per_sm,
                             bool precise, bool smem_grid, int num_sms, cudaStream_t stream,
                             int* grid_out);
// Resident CTAs per SM for a configuration (occupancy calculator).
int propagate_occupancy(int block_threads, bool precise, bool smem_tables, uint32_t blob_bytes,
                        uint32_t safety_bytes);

// Grid build on the device (pp_grid.cu).  targets_dev: n spheres in device
// memory.  Returns 0 on success; *blob_out is allocated with cudaMalloc.
int build_grid(const pp_sphere* targets_dev, int n, float cell_size, cudaStream_t stream,
               GridDev* grid_out, unsigned char** blob_out, long long* n_items_out,
               std::string* err);

// Set the calling thread's last error (pp_abi.cu); returns code.
int report_error(int code, const std::string& message);

// Grid build into caller-provided device memory (pp_grid.cu): `shape` holds
// the box, cell sizes and dims; d_counts/d_start/d_cursor have n_cells entries,
// d_totals two.  Used by the entry point that allocates nothing.
int build_grid_into(const pp_sphere* targets_dev, int n, const GridDev& shape, unsigned* d_counts,
                    unsigned* d_start, unsigned* d_cursor, unsigned* d_totals,
                    unsigned char* d_blob, size_t blob_capacity, cudaStream_t stream,
                    GridDev* grid_out, long long* n_items_out, std::string* err);
// Safety field into caller-provided device memory of shape.bytes bytes.
int build_safety_into(const pp_sphere* targets_dev, int n, const SafetyDev& shape,
                      unsigned char* d_field, cudaStream_t stream, std::string* err);

// Safety field over the grid box (pp_grid.cu); *field_out is cudaMalloc'd.
int build_safety(const pp_sphere* targets_dev, int n, const GridDev& grid, float cell,
                 cudaStream_t stream, SafetyDev* out, unsigned char** field_out, std::string* err);

// Scatter hit records into columns on the device (pp_grid.cu).
cudaError_t launch_hits_to_columns(const pp_hit_record* rec, long long n, const pp_hits& out,
                                   cudaStream_t stream);

// Philox on the device for the ABI diagnostic (pp_grid.cu).
cudaError_t launch_debug_philox(const uint32_t* ctr, int n, uint32_t k0, uint32_t k1,
                                uint32_t* out, cudaStream_t stream);

// FFMA throughput kernel (pp_grid.cu); returns flops per launch.
cudaError_t launch_fp32_peak(float* sink, int blocks, int threads, int iters, cudaStream_t stream);

}  // namespace pp
