// pp_grid.cu -- device-side build of the uniform target-culling grid, plus
// small utility kernels (hit-record transposition, Philox diagnostic, FFMA
// throughput probe).
//
// The grid replaces the reference's brute-force loop over every target in
// every step (src/photon_prop_cuda.jl:497-506): each sphere is registered in
// every cell its (slightly inflated) bounding box overlaps, so a step only
// tests the spheres of the cells its segment crosses.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "pp_device.cuh"
#include "pp_internal.h"

namespace pp {
namespace {

__device__ __forceinline__ void cell_range(const GridDev& g, const pp_sphere& t, int lo[3],
                                           int hi[3]) {
  const float r = t.radius + kGridMargin;
  for (int a = 0; a < 3; ++a) {
    int l = (int)floorf((t.position[a] - r - g.lo[a]) * g.inv_cell[a]);
    int h = (int)floorf((t.position[a] + r - g.lo[a]) * g.inv_cell[a]);
    lo[a] = max(0, min(l, g.dims[a] - 1));
    hi[a] = max(0, min(h, g.dims[a] - 1));
  }
}

// Bounding box of all inflated spheres (one CTA; n is small).
__global__ void bbox_kernel(const pp_sphere* __restrict__ t, int n, float* __restrict__ out) {
  __shared__ float red[6][256];
  float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const float r = t[i].radius + kGridMargin;
    for (int a = 0; a < 3; ++a) {
      v[a] = fminf(v[a], t[i].position[a] - r);
      v[3 + a] = fmaxf(v[3 + a], t[i].position[a] + r);
    }
  }
  for (int a = 0; a < 6; ++a) red[a][threadIdx.x] = v[a];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      for (int a = 0; a < 3; ++a) {
        red[a][threadIdx.x] = fminf(red[a][threadIdx.x], red[a][threadIdx.x + s]);
        red[3 + a][threadIdx.x] = fmaxf(red[3 + a][threadIdx.x], red[3 + a][threadIdx.x + s]);
      }
    }
    __syncthreads();
  }
  if (threadIdx.x < 6) out[threadIdx.x] = red[threadIdx.x][0];
}

__global__ void count_kernel(const GridDev g, const pp_sphere* __restrict__ t, int n,
                             unsigned* __restrict__ counts) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo[3], hi[3];
  cell_range(g, t[i], lo, hi);
  for (int z = lo[2]; z <= hi[2]; ++z)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int x = lo[0]; x <= hi[0]; ++x)
        atomicAdd(&counts[(z * g.dims[1] + y) * g.dims[0] + x], 1u);
}

// Exclusive scan of n counts in one CTA of 1024 threads: each thread scans a
// contiguous slice, the slice totals are scanned in shared memory.  Also
// reports the total and the largest count.
__global__ void scan_kernel(const unsigned* __restrict__ counts, int n, unsigned* __restrict__ start,
                            unsigned* __restrict__ totals) {
  __shared__ unsigned part[1024];
  __shared__ unsigned pmax[1024];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int b = threadIdx.x * per;
  const int e = min(n, b + per);
  unsigned s = 0, m = 0;
  for (int i = b; i < e; ++i) {
    s += counts[i];
    m = max(m, counts[i]);
  }
  part[threadIdx.x] = s;
  pmax[threadIdx.x] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned acc = 0, mm = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      const unsigned v = part[i];
      part[i] = acc;
      acc += v;
      mm = max(mm, pmax[i]);
    }
    totals[0] = acc;
    totals[1] = mm;
  }
  __syncthreads();
  unsigned acc = part[threadIdx.x];
  for (int i = b; i < e; ++i) {
    start[i] = acc;
    acc += counts[i];
  }
}

__global__ void fill_kernel(const GridDev g, const pp_sphere* __restrict__ t, int n,
                            const unsigned* __restrict__ start, unsigned* __restrict__ cursor,
                            uint16_t* __restrict__ items) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo[3], hi[3];
  cell_range(g, t[i], lo, hi);
  for (int z = lo[2]; z <= hi[2]; ++z)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int x = lo[0]; x <= hi[0]; ++x) {
        const int c = (z * g.dims[1] + y) * g.dims[0] + x;
        const unsigned slot = atomicAdd(&cursor[c], 1u);
        items[start[c] + slot] = (uint16_t)i;
      }
}

__global__ void pack_kernel(const unsigned* __restrict__ counts, const unsigned* __restrict__ start,
                            int n_cells, uint32_t* __restrict__ cells,
                            const pp_sphere* __restrict__ t, int n, float4* __restrict__ sph) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n_cells) cells[i] = (counts[i] << kCellStartBits) | (start[i] & kCellStartMask);
  if (i < n) {
    const float r = t[i].radius;
    sph[i] = make_float4(t[i].position[0], t[i].position[1], t[i].position[2], r * r);
  }
}

// One thread per safety cell: min over spheres of |c - s| - r - margin,
// floored to the quantum.  Targets are staged through shared memory.
__global__ void safety_kernel(const SafetyDev sg, const pp_sphere* __restrict__ t, int n,
                              unsigned char* __restrict__ out) {
  __shared__ float4 sh[256];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float cx = 0.0f, cy = 0.0f, cz = 0.0f;
  if (i < sg.n_cells) {
    const int x = i % sg.dims[0];
    const int y = (i / sg.dims[0]) % sg.dims[1];
    const int z = i / (sg.dims[0] * sg.dims[1]);
    cx = sg.lo[0] + (x + 0.5f) * sg.cell;
    cy = sg.lo[1] + (y + 0.5f) * sg.cell;
    cz = sg.lo[2] + (z + 0.5f) * sg.cell;
  }
  float best = 1e30f;
  for (int base = 0; base < n; base += 256) {
    const int j = base + threadIdx.x;
    __syncthreads();
    if (j < n)
      sh[threadIdx.x] = make_float4(t[j].position[0], t[j].position[1], t[j].position[2],
                                    t[j].radius + kGridMargin);
    __syncthreads();
    const int m = min(256, n - base);
    for (int k = 0; k < m; ++k) {
      const float4 s = sh[k];
      const float dx = cx - s.x, dy = cy - s.y, dz = cz - s.z;
      best = fminf(best, sqrtf(dx * dx + dy * dy + dz * dz) - s.w);
    }
  }
  if (i < sg.n_cells) {
    // 1 mm of slack covers the rounding of the distance itself
    const float q = floorf((best - 1e-3f) / kSafetyQuantum);
    out[i] = (unsigned char)fminf(fmaxf(q, 0.0f), 255.0f);
  }
}

__global__ void hits_to_columns_kernel(const pp_hit_record* __restrict__ rec, long long n,
                                       pp_hits out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const pp_hit_record h = rec[i];
  for (int a = 0; a < 3; ++a) {
    if (out.position) out.position[3 * i + a] = h.position[a];
    if (out.direction) out.direction[3 * i + a] = h.direction[a];
    if (out.initial_direction) out.initial_direction[3 * i + a] = h.initial_direction[a];
  }
  if (out.wavelength) out.wavelength[i] = h.wavelength;
  if (out.time) out.time[i] = h.time;
  if (out.dist_travelled) out.dist_travelled[i] = h.dist_travelled;
  if (out.abs_weight) out.abs_weight[i] = h.abs_weight;
  if (out.module_index) out.module_index[i] = h.module_index;
  if (out.n_steps) out.n_steps[i] = h.n_steps;
  if (out.source_index) out.source_index[i] = h.source_index;
  if (out.photon_index) out.photon_index[i] = h.photon_index;
}

__global__ void debug_philox_kernel(const uint4* __restrict__ ctr, int n, uint32_t k0, uint32_t k1,
                                    uint4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ppdev::philox(ctr[i], k0, k1);
}

// Eight independent FFMA chains per thread: the issue-limited FP32 rate.
__global__ void fp32_peak_kernel(float* __restrict__ sink, int iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
  float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.0f) sink[blockIdx.x] = s;  // keeps the chains alive
}

}  // namespace

int build_grid(const pp_sphere* targets_dev, int n, float cell_size, cudaStream_t stream,
               GridDev* grid_out, unsigned char** blob_out, long long* n_items_out,
               std::string* err) {
  auto fail = [&](const std::string& m) {
    if (err) *err = m;
    return -1;
  };
  *blob_out = nullptr;
  GridDev g{};
  if (n <= 0) {
    // Empty target list: a 1-cell grid with no items.
    g.dims[0] = g.dims[1] = g.dims[2] = 1;
    g.n_cells = 1;
    for (int a = 0; a < 3; ++a) {
      g.lo[a] = 0.0f; g.hi[a] = 1.0f; g.cell[a] = 1.0f; g.inv_cell[a] = 1.0f;
    }
    g.off_items = 16;
    g.off_spheres = 16;
    g.blob_bytes = 16;
    if (cudaMalloc(blob_out, 16) != cudaSuccess) return fail("cudaMalloc(grid blob) failed");
    if (cudaMemsetAsync(*blob_out, 0, 16, stream) != cudaSuccess) return fail("memset failed");
    *grid_out = g;
    *n_items_out = 0;
    return 0;
  }
  if (n > 65535) return fail("at most 65535 targets are supported");

  float* d_bb = nullptr;
  if (cudaMalloc(&d_bb, 6 * sizeof(float)) != cudaSuccess) return fail("cudaMalloc failed");
  bbox_kernel<<<1, 256, 0, stream>>>(targets_dev, n, d_bb);
  float bb[6];
  cudaError_t e = cudaMemcpyAsync(bb, d_bb, sizeof(bb), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  cudaFree(d_bb);
  if (e != cudaSuccess) return fail(std::string("grid bbox: ") + cudaGetErrorString(e));
  for (int a = 0; a < 6; ++a)
    if (!std::isfinite(bb[a])) return fail("target coordinates are not finite");

  double ext[3], vol = 1.0;
  for (int a = 0; a < 3; ++a) {
    ext[a] = std::max(1e-3, (double)bb[3 + a] - (double)bb[a]);
    vol *= ext[a];
  }
  double h = cell_size;
  if (!(h > 0.0)) h = std::cbrt(vol / (16.0 * n));  // about 16 cells per target
  // Keep the cell count bounded.
  const double kMaxCells = 4.0 * 1024 * 1024;
  for (int guard = 0; guard < 64; ++guard) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::max(1.0, std::ceil(ext[a] / h));
    if (cells <= kMaxCells) break;
    h *= 1.25;
  }
  for (int a = 0; a < 3; ++a) {
    g.dims[a] = (int)std::max(1.0, std::ceil(ext[a] / h));
    g.lo[a] = bb[a];
    g.cell[a] = (float)h;
    g.inv_cell[a] = (float)(1.0 / h);
    g.hi[a] = (float)((double)bb[a] + g.dims[a] * h);
  }
  g.n_cells = g.dims[0] * g.dims[1] * g.dims[2];
  g.n_targets = n;

  unsigned *d_counts = nullptr, *d_start = nullptr, *d_cursor = nullptr, *d_tot = nullptr;
  auto cleanup = [&]() {
    cudaFree(d_counts);
    cudaFree(d_start);
    cudaFree(d_cursor);
    cudaFree(d_tot);
  };
  const size_t cbytes = (size_t)g.n_cells * sizeof(unsigned);
  if (cudaMalloc(&d_counts, cbytes) != cudaSuccess || cudaMalloc(&d_start, cbytes) != cudaSuccess ||
      cudaMalloc(&d_cursor, cbytes) != cudaSuccess || cudaMalloc(&d_tot, 2 * sizeof(unsigned)) != cudaSuccess) {
    cleanup();
    return fail("cudaMalloc(grid scratch) failed");
  }
  cudaMemsetAsync(d_counts, 0, cbytes, stream);
  cudaMemsetAsync(d_cursor, 0, cbytes, stream);
  const int tb = 256;
  count_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(g, targets_dev, n, d_counts);
  scan_kernel<<<1, 1024, 0, stream>>>(d_counts, g.n_cells, d_start, d_tot);
  unsigned tot[2];
  e = cudaMemcpyAsync(tot, d_tot, sizeof(tot), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) {
    cleanup();
    return fail(std::string("grid count: ") + cudaGetErrorString(e));
  }
  const long long n_items = tot[0];
  if (n_items > (long long)kCellStartMask || tot[1] > kCellMaxCount) {
    cleanup();
    char buf[200];
    snprintf(buf, sizeof(buf),
             "grid too dense (%lld items, %u in one cell): choose a smaller cell size", n_items,
             tot[1]);
    return fail(buf);
  }
  auto pad16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  const size_t cells_b = pad16(cbytes);
  const size_t items_b = pad16((size_t)std::max<long long>(n_items, 1) * sizeof(uint16_t));
  const size_t sph_b = (size_t)n * sizeof(float4);
  g.off_items = (uint32_t)cells_b;
  g.off_spheres = (uint32_t)(cells_b + items_b);
  const size_t total = cells_b + items_b + sph_b;
  if (total > 0xffffffffull) {
    cleanup();
    return fail("grid blob larger than 4 GiB");
  }
  g.blob_bytes = (uint32_t)total;
  unsigned char* blob = nullptr;
  if (cudaMalloc(&blob, total) != cudaSuccess) {
    cleanup();
    return fail("cudaMalloc(grid blob) failed");
  }
  cudaMemsetAsync(blob, 0, total, stream);
  fill_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(g, targets_dev, n, d_start, d_cursor,
                                                   reinterpret_cast<uint16_t*>(blob + g.off_items));
  const int m = std::max(g.n_cells, n);
  pack_kernel<<<(m + tb - 1) / tb, tb, 0, stream>>>(
      d_counts, d_start, g.n_cells, reinterpret_cast<uint32_t*>(blob), targets_dev, n,
      reinterpret_cast<float4*>(blob + g.off_spheres));
  e = cudaStreamSynchronize(stream);
  cleanup();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(blob);
    return fail(std::string("grid build: ") + cudaGetErrorString(e));
  }
  *grid_out = g;
  *blob_out = blob;
  *n_items_out = n_items;
  return 0;
}

int build_safety(const pp_sphere* targets_dev, int n, const GridDev& grid, float cell,
                 cudaStream_t stream, SafetyDev* out, unsigned char** field_out, std::string* err) {
  *field_out = nullptr;
  SafetyDev sg{};
  double h = cell > 0.0f ? cell : 12.5;
  double ext[3];
  for (int a = 0; a < 3; ++a) ext[a] = (double)grid.hi[a] - (double)grid.lo[a];
  for (int guard = 0; guard < 64; ++guard) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) cells *= std::max(1.0, std::ceil(ext[a] / h));
    if (cells <= 16.0 * 1024 * 1024) break;
    h *= 1.25;
  }
  sg.n_cells = 1;
  for (int a = 0; a < 3; ++a) {
    sg.dims[a] = (int)std::max(1.0, std::ceil(ext[a] / h));
    sg.lo[a] = grid.lo[a];
    sg.hi[a] = (float)((double)grid.lo[a] + sg.dims[a] * h);
    sg.n_cells *= sg.dims[a];
  }
  sg.cell = (float)h;
  sg.inv_cell = (float)(1.0 / h);
  sg.bytes = (uint32_t)(((size_t)sg.n_cells + 15) & ~(size_t)15);
  sg.set_derived();
  unsigned char* f = nullptr;
  if (cudaMalloc(&f, (size_t)sg.bytes) != cudaSuccess) {
    if (err) *err = "cudaMalloc(safety field) failed";
    return -1;
  }
  cudaMemsetAsync(f, 0, (size_t)sg.bytes, stream);
  if (n <= 0) {
    cudaMemsetAsync(f, 255, (size_t)sg.n_cells, stream);
  } else {
    safety_kernel<<<(sg.n_cells + 255) / 256, 256, 0, stream>>>(sg, targets_dev, n, f);
  }
  cudaError_t e = cudaStreamSynchronize(stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(f);
    if (err) *err = std::string("safety field: ") + cudaGetErrorString(e);
    return -1;
  }
  *out = sg;
  *field_out = f;
  return 0;
}

int build_grid_into(const pp_sphere* targets_dev, int n, const GridDev& shape, unsigned* d_counts,
                    unsigned* d_start, unsigned* d_cursor, unsigned* d_totals,
                    unsigned char* d_blob, size_t blob_capacity, cudaStream_t stream,
                    GridDev* grid_out, long long* n_items_out, std::string* err) {
  auto fail = [&](const std::string& m) {
    if (err) *err = m;
    return -1;
  };
  GridDev g = shape;
  const size_t cbytes = (size_t)g.n_cells * sizeof(unsigned);
  cudaMemsetAsync(d_counts, 0, cbytes, stream);
  cudaMemsetAsync(d_cursor, 0, cbytes, stream);
  const int tb = 256;
  if (n > 0) count_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(g, targets_dev, n, d_counts);
  scan_kernel<<<1, 1024, 0, stream>>>(d_counts, g.n_cells, d_start, d_totals);
  unsigned tot[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(tot, d_totals, sizeof(tot), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return fail(std::string("grid count: ") + cudaGetErrorString(e));
  const long long n_items = tot[0];
  if (n_items > (long long)kCellStartMask || tot[1] > kCellMaxCount)
    return fail("grid too dense: choose a smaller cell size");
  auto pad16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  const size_t cells_b = pad16(cbytes);
  const size_t items_b = pad16((size_t)std::max<long long>(n_items, 1) * sizeof(uint16_t));
  const size_t total = cells_b + items_b + (size_t)n * sizeof(float4);
  if (total > blob_capacity) return fail("grid larger than the space reserved for it");
  g.off_items = (uint32_t)cells_b;
  g.off_spheres = (uint32_t)(cells_b + items_b);
  g.blob_bytes = (uint32_t)total;
  g.n_targets = n;
  cudaMemsetAsync(d_blob, 0, total, stream);
  if (n > 0)
    fill_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(g, targets_dev, n, d_start, d_cursor,
                                                     reinterpret_cast<uint16_t*>(d_blob + g.off_items));
  const int m = std::max(g.n_cells, n);
  pack_kernel<<<(m + tb - 1) / tb, tb, 0, stream>>>(
      d_counts, d_start, g.n_cells, reinterpret_cast<uint32_t*>(d_blob), targets_dev, n,
      reinterpret_cast<float4*>(d_blob + g.off_spheres));
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(std::string("grid build: ") + cudaGetErrorString(e));
  *grid_out = g;
  *n_items_out = n_items;
  return 0;
}

int build_safety_into(const pp_sphere* targets_dev, int n, const SafetyDev& shape,
                      unsigned char* d_field, cudaStream_t stream, std::string* err) {
  cudaMemsetAsync(d_field, 0, (size_t)shape.bytes, stream);
  if (n <= 0) {
    cudaMemsetAsync(d_field, 255, (size_t)shape.n_cells, stream);
  } else {
    safety_kernel<<<(shape.n_cells + 255) / 256, 256, 0, stream>>>(shape, targets_dev, n, d_field);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    if (err) *err = std::string("safety field: ") + cudaGetErrorString(e);
    return -1;
  }
  return 0;
}

cudaError_t launch_hits_to_columns(const pp_hit_record* rec, long long n, const pp_hits& out,
                                   cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int tb = 256;
  const long long blocks = (n + tb - 1) / tb;
  hits_to_columns_kernel<<<(unsigned)blocks, tb, 0, stream>>>(rec, n, out);
  return cudaGetLastError();
}

cudaError_t launch_debug_philox(const uint32_t* ctr, int n, uint32_t k0, uint32_t k1,
                                uint32_t* out, cudaStream_t stream) {
  const int tb = 128;
  debug_philox_kernel<<<(n + tb - 1) / tb, tb, 0, stream>>>(reinterpret_cast<const uint4*>(ctr), n,
                                                          k0, k1, reinterpret_cast<uint4*>(out));
  return cudaGetLastError();
}

cudaError_t launch_fp32_peak(float* sink, int blocks, int threads, int iters, cudaStream_t stream) {
  fp32_peak_kernel<<<blocks, threads, 0, stream>>>(sink, iters);
  return cudaGetLastError();
}

}  // namespace pp
