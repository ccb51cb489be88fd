// pp_propagate.cu -- fast variant of the propagation kernel and the host-side
// launch (grid sizing from the occupancy calculator, dynamic shared memory for
// the staged target grid).
#include <cuda_runtime.h>

#include "pp_kernel.cuh"

namespace pp {

// Replay variant, instantiated in pp_propagate_precise.cu.
const void* precise_kernel_ptr(bool smem_grid, bool shapes);

namespace {

const void* select_kernel(bool precise, bool smem_grid, bool shapes = false) {
  if (precise) return precise_kernel_ptr(smem_grid, shapes);
  if (shapes) return kernel_ptr<false, false, true>();
  return smem_grid ? kernel_ptr<false, true>() : kernel_ptr<false, false>();
}

}  // namespace

int propagate_occupancy(int block_threads, bool precise, bool smem_tables, uint32_t blob_bytes,
                        uint32_t safety_bytes) {
  const void* k = select_kernel(precise, smem_tables);
  const size_t smem_bytes = propagate_smem_bytes(blob_bytes, safety_bytes, smem_tables,
                                                 block_threads, nullptr, nullptr);
  if (smem_bytes > 48 * 1024)
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block_threads, smem_bytes) != cudaSuccess)
    return 0;
  return n;
}

cudaError_t launch_propagate(const LaunchArgs& args, int block_threads, int ctas_per_sm,
                             bool precise, bool smem_grid, int num_sms, cudaStream_t stream,
                             int* grid_out) {
  const bool shapes = args.shapes != nullptr;
  if (shapes) smem_grid = false;
  const void* k = select_kernel(precise, smem_grid, shapes);
  if (block_threads > kMaxBlockThreads || block_threads % 32) return cudaErrorInvalidValue;
  LaunchArgs a = args;
  const size_t smem = propagate_smem_bytes(args.grid.blob_bytes, args.sgrid.bytes, smem_grid,
                                           block_threads, &a.safety_offset, &a.state_offset);
  a.warps_per_block = block_threads / 32;
  cudaError_t e;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, block_threads, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int per_sm = ctas_per_sm > 0 ? (ctas_per_sm < occ ? ctas_per_sm : occ) : occ;
  int grid = per_sm * num_sms;
  // Never launch more warps than there are chunks of work.
  const unsigned long long warps_per_cta = (unsigned long long)(block_threads / 32);
  const unsigned long long need = (args.total_chunks + warps_per_cta - 1) / warps_per_cta;
  if (need < (unsigned long long)grid) grid = (int)(need > 0 ? need : 1);
  if (grid_out) *grid_out = grid;
  void* params[] = {&a};
  return cudaLaunchKernel(k, dim3(grid), dim3(block_threads), params, smem, stream);
}

}  // namespace pp
