// pp_propagate_precise.cu -- replay variant of the propagation kernel.
//
// Built with -fmad=false: no multiply-add contraction, so each FP32
// expression written in the same form as the CPU oracle's rounds the same way;
// transcendental functions come from the IEEE-accurate CUDA math library.
// Used to check trajectories photon by photon against the oracle.
#include <cuda_runtime.h>

#include "pp_kernel.cuh"

namespace pp {

const void* precise_kernel_ptr(bool smem_grid, bool shapes) {
  if (shapes) return kernel_ptr<true, false, true>();
  return smem_grid ? kernel_ptr<true, true>() : kernel_ptr<true, false>();
}

}  // namespace pp
