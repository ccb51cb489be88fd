// pp_mlp.cu -- the learned surrogate: a small MLP trained and evaluated with
// hand-written tcgen05 kernels (BF16 operands, FP32 accumulation in tensor
// memory) for training and for the fused inference kernel.
//
// No counterpart in the reference: PhotonPropagation.jl evaluates an external
// surrogate (PhotonSurrogateModel, examples/validation.jl:455,673-676) whose
// weights are not part of the repository.  Here the network maps
// source-module geometry to the expected hit count and a 64-bin arrival-time
// distribution, trained on tables the MC kernel generates
// (pp_launch_histogram).
//
// Network: x (n_in, zero-padded to a multiple of 16) -> 4 x [256, SiLU] ->
// head (1 log-expected-count + 64 time logits, padded to 80).  Loss per sample
// (Poisson + multinomial negative log-likelihood):
//   L = exp(o0) - k*o0 - sum_b h_b * log softmax(o_1..64)_b.
// Parameters are FP32 masters with a BF16 copy for training and a BF16 pack
// in the tensor core's layout for inference; Adam.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "pp_device.cuh"
#include "pp_internal.h"
#include "pp_tc.cuh"

using bf16 = __nv_bfloat16;

namespace {

constexpr int kTileM = 128;   // rows per CTA tile (tcgen05 M)
constexpr int kKC = 64;       // K columns staged per iteration
constexpr int kGemmThreads = 256;  // two warps per TMEM lane quarter
constexpr unsigned long long kWaitNs = 1000000000ull;

enum GemmMode : int {
  kStoreF32 = 0,     // C32 = acc + bias
  kHiddenFwd = 1,    // Z16 = acc + bias, C16 = silu(acc + bias)
  kBackwardDx = 2,   // C16 = acc * silu'(Zprev)
  kAccumulateF32 = 3 // C32 += acc (atomic, split-K)
};

struct GemmParams {
  const bf16* A;
  long long lda;
  int a_trans;  // element (m, k) = a_trans ? A[k*lda + m] : A[m*lda + k]
  const bf16* B;
  long long ldb;
  int b_trans;  // element (n, k) = b_trans ? B[k*ldb + n] : B[n*ldb + k]
  int M, N, K;  // N <= 256 and N % 16 == 0; K % 16 == 0
  int k_per_split;
  int mode;
  const float* bias;
  float* C32;
  long long ldc;
  bf16* C16;
  long long ldc16;
  bf16* Z16;
  long long ldz;
  const bf16* Zprev;
  long long ldzp;
  unsigned* err;
};

__host__ __device__ inline uint32_t tmem_cols_for(int n) {
  uint32_t c = 32;
  while (c < (uint32_t)n) c <<= 1;
  return c;
}

// Prologue of every kernel of the training step.  The step's kernels are
// launched with programmatic stream serialisation (launch_pdl), so a kernel's
// blocks may be scheduled while its predecessor in the stream still runs:
// griddepcontrol.wait holds them until the predecessor has completed and its
// writes are visible (a no-op for a kernel launched without the attribute),
// and launch_dependents then lets the next kernel be scheduled.  Nothing
// before pdl_begin may read what an earlier kernel of the stream wrote.
__device__ __forceinline__ void pdl_begin() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Training GEMM.  One CTA computes a kTileM x (<= kTileN) tile of
// D = A * B^T over at most kGemmStages * kKC of K (longer reductions are split
// over blockIdx.z and accumulated atomically).  Every K stage of both operands
// is requested at once with 16-byte cp.async copies straight into the tensor
// core's core-matrix layout (no register round trip, zero-filled past the
// edges); the MMAs of a stage are issued as soon as it lands.  Eight warps:
// warps w and w + 4 read TMEM lane quarter w % 4 (rows 32 (w % 4) .. + 31 of
// the tile) and take alternate 32-column slices of the accumulator, so that
// two warps per scheduler hide each other's latency in the copy issue and the
// epilogue.
//
// Shared-memory tile of R rows (M or N) x kKC columns of K, 8 x 8 core matrices
// of 128 bytes, core matrix (r / 8, k / 8) at ((r / 8) * (kKC / 8) + k / 8) * 128:
//   K-major  (operand stored row-major over K): row r%8 at +16 (r%8), k%8 at +2 (k%8);
//   MN-major (operand stored with R contiguous, a_trans / b_trans): k%8 at +16 (k%8),
//            r%8 at +2 (r%8), and the instruction descriptor's transpose bit set.
// Without swizzling both use the descriptor's LBO for the stride between core
// matrices along K (128 B) and SBO for the stride along R (1024 B).  Either
// way a 16-byte piece (8 consecutive elements of the contiguous dimension) is
// one contiguous 16-byte row of a core matrix, and a K step of 16 advances the
// descriptor by 256 bytes.
// (A 128 x 64 tile, two CTAs per SM at 96 KB each, measured 8 % slower per
// training step: per-CTA setup and the re-read A tiles outweigh the overlap.)
constexpr int kTileN = 128;
constexpr int kGemmStages = 4;                          // K <= 256 per CTA
constexpr uint32_t kTileBytes = kTileM * kKC * 2u;      // the A tile of one stage
constexpr uint32_t kTileBytesB = kTileN * kKC * 2u;     // the B tile of one stage
constexpr uint32_t kStageBytes = kTileBytes + kTileBytesB;

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_pending(int n) {  // n in 0..kGemmStages-1
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
  }
}

// Request rows [r0, r0 + rows_tile) x K [k0, k0 + kKC) of one operand.
__device__ __forceinline__ void stage_async(uint32_t dst, const bf16* __restrict__ src,
                                            long long ld, int trans, int r0, int rows_valid,
                                            int rows_tile, int k0, int kend) {
  const int pieces = rows_tile * (kKC / 8);
  for (int c = threadIdx.x; c < pieces; c += blockDim.x) {
    uint32_t off, bytes;
    const bf16* g;
    if (!trans) {  // piece = row r, K elements 8 kb .. 8 kb + 7
      const int r = c >> 3, kb = c & 7;
      const int k = k0 + kb * 8;
      const bool in = r < rows_valid && k < kend;
      off = (uint32_t)(((r >> 3) * (kKC / 8) + kb) * 128 + (r & 7) * 16);
      g = in ? src + (long long)(r0 + r) * ld + k : src;
      bytes = in ? 16u : 0u;
    } else {       // piece = K element k, rows 8 g .. 8 g + 7
      const int k = c % kKC, gr = c / kKC;
      const int left = rows_valid - gr * 8;
      const bool in = k0 + k < kend && left > 0;
      off = (uint32_t)((gr * (kKC / 8) + (k >> 3)) * 128 + (k & 7) * 16);
      g = in ? src + (long long)(k0 + k) * ld + r0 + gr * 8 : src;
      bytes = in ? (uint32_t)(left >= 8 ? 16 : 2 * left) : 0u;
    }
    cp_async16(dst + off, g, bytes);
  }
}

__global__ void __launch_bounds__(kGemmThreads) gemm_kernel(const __grid_constant__ GemmParams p) {
  pdl_begin();
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * kTileM;
  const int n0 = blockIdx.y * kTileN;
  const int nt = min(kTileN, p.N - n0);  // multiple of 16
  const int kbeg = blockIdx.z * p.k_per_split;
  const int kend = min(p.K, kbeg + p.k_per_split);
  const int nk = (kend - kbeg + kKC - 1) / kKC;  // <= kGemmStages
  const uint32_t ncols = tmem_cols_for(nt);
  const uint32_t s0 = pptc::smem_u32(smem);

  for (int st = 0; st < nk; ++st) {
    const int k0 = kbeg + st * kKC;
    stage_async(s0 + st * kStageBytes, p.A, p.lda, p.a_trans, m0, min(kTileM, p.M - m0), kTileM,
                k0, kend);
    stage_async(s0 + st * kStageBytes + kTileBytes, p.B + (p.b_trans ? n0 : (long long)n0 * p.ldb),
                p.ldb, p.b_trans, 0, nt, nt, k0, kend);
    cp_async_commit();
  }
  if (warp == 0) pptc::tmem_alloc(&tmem_slot, ncols);
  if (threadIdx.x == 0) pptc::mbar_init(&bar, 1);
  pptc::fence_before_sync();
  __syncthreads();
  pptc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = pptc::idesc_bf16(kTileM, nt) | ((uint32_t)(p.a_trans != 0) << 15) |
                         ((uint32_t)(p.b_trans != 0) << 16);

  for (int st = 0; st < nk; ++st) {
    cp_async_wait_pending(nk - 1 - st);  // this thread's copies of stage st have landed
    pptc::fence_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
      pptc::fence_after_sync();
      const uint32_t sa = s0 + st * kStageBytes, sb = sa + kTileBytes;
      const int k0 = kbeg + st * kKC;
      for (int s = 0; s < kKC / 16 && k0 + s * 16 < kend; ++s) {
        const uint64_t ad = pptc::smem_desc(sa + s * 256, 128, 1024);
        const uint64_t bd = pptc::smem_desc(sb + s * 256, 128, 1024);
        pptc::mma_f16(tmem, ad, bd, idesc, st > 0 || s > 0);
      }
    }
  }
  if (threadIdx.x == 0) pptc::mma_commit(&bar);
  // this thread's row, and its (at most two) 32-column slices c0 = 32 (warp / 4)
  // + 64 si; for the backward dX, the row's saved pre-activations of those
  // slices are loaded here, while the MMAs run
  const int quarter = warp & 3;
  const int row = m0 + quarter * 32 + lane;
  const bool row_ok = row < p.M;
  uint4 zpre[2][4];
  if (p.mode == kBackwardDx && row_ok && nk > 0) {
#pragma unroll
    for (int si = 0; si < 2; ++si)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int cc = (warp >> 2) * 32 + si * 64 + q * 8;
        if (cc < nt)
          zpre[si][q] =
              __ldg(reinterpret_cast<const uint4*>(p.Zprev + (long long)row * p.ldzp + n0 + cc));
      }
  }
  bool ok = nk > 0 ? pptc::mbar_wait(&bar, 0, kWaitNs) : true;
  ok = __syncthreads_and(ok);
  pptc::fence_after_sync();

  if (ok && nk > 0) {
#pragma unroll
    for (int si = 0; si < 2; ++si) {
      const int c0 = (warp >> 2) * 32 + si * 64;
      if (c0 >= nt) break;
      float v[32];
      pptc::tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
      if (!row_ok) continue;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int col = n0 + c0 + q * 8;  // 8 columns per 16-byte group
        if (c0 + q * 8 >= nt) break;
        const float* a8 = v + q * 8;
        switch (p.mode) {
          case kStoreF32: {
            float4 lo = make_float4(a8[0], a8[1], a8[2], a8[3]);
            float4 hi = make_float4(a8[4], a8[5], a8[6], a8[7]);
            if (p.bias) {
              const float4 b0 = __ldg(reinterpret_cast<const float4*>(p.bias + col));
              const float4 b1 = __ldg(reinterpret_cast<const float4*>(p.bias + col + 4));
              lo.x += b0.x; lo.y += b0.y; lo.z += b0.z; lo.w += b0.w;
              hi.x += b1.x; hi.y += b1.y; hi.z += b1.z; hi.w += b1.w;
            }
            float4* d = reinterpret_cast<float4*>(p.C32 + (long long)row * p.ldc + col);
            d[0] = lo;
            d[1] = hi;
            break;
          }
          case kHiddenFwd: {
            const float4 b0 = __ldg(reinterpret_cast<const float4*>(p.bias + col));
            const float4 b1 = __ldg(reinterpret_cast<const float4*>(p.bias + col + 4));
            const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            union {
              uint4 u4;
              __nv_bfloat162 h2[4];
            } z16, y16;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float za = a8[2 * j] + bb[2 * j], zb = a8[2 * j + 1] + bb[2 * j + 1];
              z16.h2[j] = __floats2bfloat162_rn(za, zb);
              y16.h2[j] = __floats2bfloat162_rn(pptc::silu(za), pptc::silu(zb));
            }
            *reinterpret_cast<uint4*>(p.Z16 + (long long)row * p.ldz + col) = z16.u4;
            *reinterpret_cast<uint4*>(p.C16 + (long long)row * p.ldc16 + col) = y16.u4;
            break;
          }
          case kBackwardDx: {
            union {
              uint4 u4;
              __nv_bfloat162 h2[4];
            } zp, o;
            zp.u4 = zpre[si][q];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float2 z = __bfloat1622float2(zp.h2[j]);
              o.h2[j] = __floats2bfloat162_rn(a8[2 * j] * pptc::silu_grad(z.x),
                                              a8[2 * j + 1] * pptc::silu_grad(z.y));
            }
            *reinterpret_cast<uint4*>(p.C16 + (long long)row * p.ldc16 + col) = o.u4;
            break;
          }
          default: {
            float4* d = reinterpret_cast<float4*>(p.C32 + (long long)row * p.ldc + col);
            atomicAdd(d, make_float4(a8[0], a8[1], a8[2], a8[3]));
            atomicAdd(d + 1, make_float4(a8[4], a8[5], a8[6], a8[7]));
            break;
          }
        }
      }
    }
  }
  cp_async_wait_pending(0);  // nothing in flight when shared memory is released
  pptc::fence_before_sync();
  __syncthreads();
  if (warp == 0) pptc::tmem_dealloc(tmem, ncols);
  if (!ok && threadIdx.x == 0) atomicOr(p.err, 1u);
}

// Features (n x n_in, FP32) -> zero-padded BF16 rows of in_pad.
__global__ void pack_input_kernel(const float* __restrict__ x, int n, int n_in, int in_pad,
                                  bf16* __restrict__ out) {
  pdl_begin();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)n * in_pad) return;
  const long long r = i / in_pad;
  const int c = (int)(i % in_pad);
  out[i] = __float2bfloat16(c < n_in ? x[r * n_in + c] : 0.0f);
}

// Poisson + multinomial NLL per sample (one warp per sample) and its gradient
// with respect to the head outputs.
// Poisson + multinomial loss of a batch and its gradient with respect to the
// head's outputs, one warp per row in one pass: the row's logits and
// histogram stay in registers (bin j = lane + 32 i, n_bins <= kLossBinsPerLane
// * 32).  Writes dO16 (BF16, every column up to out_pad, zero past the last
// bin) and adds the rows' sums of the FP32 gradient into gbias (the head's
// bias gradient) and their losses into *loss, once per block.
constexpr int kLossBinsPerLane = 8;
constexpr int kLossWarps = 8;
__global__ void __launch_bounds__(kLossWarps * 32)
    loss_kernel(const float* __restrict__ O, long long ldo, int B, const float* __restrict__ count,
                const float* __restrict__ hist, int nb, float inv_b, float time_weight,
                bf16* __restrict__ dO16, long long ldd, int out_pad, float* __restrict__ gbias,
                float* __restrict__ loss) {
  pdl_begin();
  __shared__ float s_g[kLossWarps][kLossBinsPerLane * 32 + 1];
  __shared__ float s_loss[kLossWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float gsum[kLossBinsPerLane + 1];  // [i]: column 1 + lane + 32 i; [last]: column 0
#pragma unroll
  for (int i = 0; i <= kLossBinsPerLane; ++i) gsum[i] = 0.0f;
  float lsum = 0.0f;
  for (int row = blockIdx.x * kLossWarps + warp; row < B; row += gridDim.x * kLossWarps) {
    const float* o = O + (long long)row * ldo;
    const float* h = hist + (long long)row * nb;
    float x[kLossBinsPerLane], hv[kLossBinsPerLane];
    float mx = -INFINITY;
#pragma unroll
    for (int i = 0; i < kLossBinsPerLane; ++i) {
      const int j = lane + 32 * i;
      x[i] = j < nb ? __ldg(o + 1 + j) : -INFINITY;
      hv[i] = j < nb ? __ldg(h + j) : 0.0f;
      mx = fmaxf(mx, x[i]);
    }
    for (int sh = 16; sh > 0; sh >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, sh));
    float se = 0.0f, hs = 0.0f, hx = 0.0f;
#pragma unroll
    for (int i = 0; i < kLossBinsPerLane; ++i) {
      if (lane + 32 * i < nb) {
        x[i] -= mx;
        hs += hv[i];
        hx += hv[i] * x[i];
        x[i] = __expf(x[i]);  // from here on the unnormalised probability
        se += x[i];
      }
    }
    for (int sh = 16; sh > 0; sh >>= 1) {
      se += __shfl_xor_sync(0xffffffffu, se, sh);
      hs += __shfl_xor_sync(0xffffffffu, hs, sh);
      hx += __shfl_xor_sync(0xffffffffu, hx, sh);
    }
    const float inv_se = 1.0f / se;
    const float gw = inv_b * time_weight;
    bf16* d16 = dO16 + (long long)row * ldd;
#pragma unroll
    for (int i = 0; i < kLossBinsPerLane; ++i) {
      const int col = 1 + lane + 32 * i;
      if (col < out_pad) {
        const float g = col - 1 < nb ? (hs * (x[i] * inv_se) - hv[i]) * gw : 0.0f;
        d16[col] = __float2bfloat16(g);
        gsum[i] += g;
      }
    }
    if (lane == 0) {
      const float o0 = fminf(o[0], 30.0f);
      const float lam = __expf(o0);
      const float k = count[row];
      const float g0 = (lam - k) * inv_b;
      d16[0] = __float2bfloat16(g0);
      gsum[kLossBinsPerLane] += g0;
      const float lt = -(hx - hs * __logf(se));
      lsum += (lam - k * o0 + time_weight * lt) * inv_b;
    }
  }
#pragma unroll
  for (int i = 0; i < kLossBinsPerLane; ++i) s_g[warp][1 + lane + 32 * i] = gsum[i];
  if (lane == 0) {
    s_g[warp][0] = gsum[kLossBinsPerLane];
    s_loss[warp] = lsum;
  }
  __syncthreads();
  for (int col = threadIdx.x; col < out_pad; col += blockDim.x) {
    float t = 0.0f;
#pragma unroll
    for (int w = 0; w < kLossWarps; ++w) t += s_g[w][col];
    atomicAdd(gbias + col, t);
  }
  if (threadIdx.x == 0) {
    float t = 0.0f;
#pragma unroll
    for (int w = 0; w < kLossWarps; ++w) t += s_loss[w];
    atomicAdd(loss, t);
  }
}

// out[c] += sum over rows of X[r][c] for the BF16 gradients of a hidden layer
// (bias gradients): lane l of each warp sums columns 8 l .. 8 l + 7 with
// 16-byte loads over the warp's rows, the block's warps meet in shared memory
// and add once per column.  cols <= 256 and a multiple of 8, ld a multiple of
// 8, X 16-byte aligned.
constexpr int kColsumWarps = 8;
__global__ void __launch_bounds__(kColsumWarps * 32)
    colsum_kernel(const bf16* __restrict__ X, int rows, int cols, long long ld,
                  float* __restrict__ out) {
  pdl_begin();
  __shared__ float red[kColsumWarps][257];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = lane * 8;
  float acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = 0.0f;
  if (c < cols) {
    for (int r = blockIdx.x * kColsumWarps + warp; r < rows; r += gridDim.x * kColsumWarps) {
      union {
        uint4 u4;
        __nv_bfloat162 h2[4];
      } v;
      v.u4 = __ldg(reinterpret_cast<const uint4*>(X + (long long)r * ld + c));
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float2 f = __bfloat1622float2(v.h2[j]);
        acc[2 * j] += f.x;
        acc[2 * j + 1] += f.y;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 8; ++j) red[warp][c + j] = acc[j];
  __syncthreads();
  for (int col = threadIdx.x; col < cols; col += blockDim.x) {
    float t = 0.0f;
#pragma unroll
    for (int w = 0; w < kColsumWarps; ++w) t += red[w][col];
    atomicAdd(out + col, t);
  }
}

__global__ void adam_kernel(float* __restrict__ w, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, long long n, float lr,
                            float b1, float b2, float eps, float bc1, float bc2,
                            bf16* __restrict__ w16) {
  pdl_begin();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  w16[i] = __float2bfloat16(wi);
}

// Adam with its step size and bias corrections read from device memory
// (sched[0..2], written by schedule_kernel), for the captured training step.
__global__ void adam_dev_kernel(float* __restrict__ w, const float* __restrict__ g,
                                float* __restrict__ m, float* __restrict__ v, long long n,
                                const float* __restrict__ sched, float b1, float b2, float eps,
                                bf16* __restrict__ w16) {
  pdl_begin();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float lr = sched[0], bc1 = sched[1], bc2 = sched[2];
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  const float wi = w[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  w[i] = wi;
  w16[i] = __float2bfloat16(wi);
}

// The step about to be taken (Adam step t = *step + 1): its cosine step size
// and bias corrections, in double and rounded once, as pp_mlp_train_step
// computes them.
__global__ void schedule_kernel(const long long* __restrict__ step, long long step0,
                                long long total, float lr0, float lr1, float b1, float b2,
                                float* __restrict__ sched) {
  pdl_begin();
  const long long done = *step;
  const double frac = total > 1 ? (double)(done - step0) / (double)(total - 1) : 0.0;
  sched[0] = (float)((double)lr1 + 0.5 * ((double)lr0 - (double)lr1) *
                                       (1.0 + cos(3.14159265358979323846 * frac)));
  sched[1] = (float)(1.0 - pow((double)b1, (double)(done + 1)));
  sched[2] = (float)(1.0 - pow((double)b2, (double)(done + 1)));
}

__global__ void step_kernel(long long* step) {
  pdl_begin();
  *step += 1;
}

// Zero the gradient accumulator and the loss (a kernel rather than a memset,
// so that the step's launches stay one programmatic chain).
__global__ void zero_kernel(float* __restrict__ g, long long n, float* __restrict__ loss) {
  pdl_begin();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) g[i] = 0.0f;
  if (i == 0) *loss = 0.0f;
}
__global__ void set_step_kernel(long long* step, long long v) { *step = v; }

// Batch row i of Adam step t = *step + 1: training row
// floor(Philox(i, t, tag) * n_rows / 2^64), one warp per batch row.
constexpr uint32_t kBatchTag = 0x42415443u;  // Philox counter word of the batch stream
__global__ void gather_kernel(const float* __restrict__ x, const float* __restrict__ c,
                              const float* __restrict__ h, long long n_rows, int n_in,
                              int n_bins, int B, const long long* __restrict__ step,
                              uint32_t k0, uint32_t k1, float* __restrict__ bx,
                              float* __restrict__ bc, float* __restrict__ bh) {
  pdl_begin();
  const int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= B) return;
  const unsigned long long t = (unsigned long long)(*step + 1);
  const uint4 r = ppdev::philox(make_uint4((uint32_t)i, (uint32_t)t, (uint32_t)(t >> 32), kBatchTag),
                                k0, k1);
  const unsigned long long u = ((unsigned long long)r.x << 32) | r.y;
  const long long row = (long long)__umul64hi(u, (unsigned long long)n_rows);
  for (int j = lane; j < n_in; j += 32) bx[(long long)i * n_in + j] = x[row * n_in + j];
  for (int j = lane; j < n_bins; j += 32) bh[(long long)i * n_bins + j] = h[row * n_bins + j];
  if (lane == 0) bc[i] = c[row];
}

__global__ void to_bf16_kernel(const float* __restrict__ x, long long n, bf16* __restrict__ y) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16(x[i]);
}

// ---------------------------------------------------------------------------
// Fused inference.
//
// The inference network runs in BF16 (BF16 operands and activations, FP32
// accumulators and FP32 bias + SiLU), the rounding points of the training
// forward pass.  BF16 keeps FP32's exponent range, so no activation can
// overflow.  Weights are
// packed once per parameter update from the FP32 parameters, the hidden
// layers' scaled by 1/2 (exact in BF16) so that the accumulator is z/2 - b/2
// (h = z/2 is the argument of silu(z) = h + h tanh(h)), into K-chunks of
// kChunkK columns (the
// last chunk of a layer may be 16 wide), each chunk a contiguous block in the
// tensor core's core-matrix layout: element (r, c) of layer l (rows x cols) at
//   wpack_off[l] + (c / kChunkK) * rows * kChunkK * 2
//   + core_offset(r, (c % kChunkK) / 8, chunk width) + (c % 8) * 2,
// so that one TMA bulk copy brings one chunk into a ring slot.
constexpr int kChunkK = 64;
constexpr int kRingSlots = 3;
constexpr uint32_t kSlotBytes = 256u * kChunkK * 2u;  // up to 256 rows x 64 16-bit values
constexpr uint32_t kRedBytes = 2u * 4u * 128u * 4u;   // head: row max and sum per column group
// one-pass head: max and sum per 16-column half and row, then the halves' scales
constexpr uint32_t kHeadRedBytes = 3u * 8u * 128u * 4u;

__host__ __device__ inline int chunk_width(int K, int j) {
  return K - j * kChunkK < kChunkK ? K - j * kChunkK : kChunkK;
}

__global__ void repack_kernel(const float* __restrict__ w, int rows, int cols, float scale,
                              unsigned char* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)rows * cols) return;
  const int r = (int)(i / cols), c = (int)(i % cols);
  const int j = c / kChunkK, cc = c % kChunkK;
  const size_t off = (size_t)j * rows * kChunkK * 2 +
                     pptc::core_offset(r, cc >> 3, chunk_width(cols, j)) + (cc & 7) * 2;
  *reinterpret_cast<bf16*>(out + off) = __float2bfloat16_rn(w[i] * scale);
}

constexpr int kMaxLayers = 17;
constexpr size_t kMaxInferSmem = 232448 - 256;  // 227 KB opt-in less the static barriers
constexpr int kEpiWarps = 16;                        // epilogue warps (4 per TMEM lane quarter)
constexpr int kEpiThreads = kEpiWarps * 32;
constexpr int kInferThreads = 64 + kEpiThreads;      // producer warp, MMA warp, epilogue
struct InferParams {
  const float* x;
  long long n;
  int n_in, in_pad, hidden, n_layers, out_pad, n_bins;
  int n_tiles, n_rounds;
  uint32_t slot_cols;               // TMEM columns per accumulator (power of two >= 32)
  uint32_t act_bytes;               // one tile's activations (128 x max(in_pad, hidden) BF16)
  uint32_t ring_off;                // shared-memory byte offset of the weight ring
  uint32_t head_bias_off;           // offset of the head's FP32 biases (one-pass head), or 0
  int stage_pdf;                    // PDF rows staged through shared memory
  const unsigned char* wpack;
  long long wpack_off[kMaxLayers];  // bytes, multiples of 512
  const float* P;                   // FP32 parameters (the head's biases)
  long long off_b[kMaxLayers];
  float* expect;                    // [n]
  float* pdf;                       // [n x n_bins], may be null
  unsigned* err;
  unsigned long long wait_ns;       // bound on every mbarrier wait
  int skip_first_copy;              // diagnostic: chunk 0's barrier armed, no copy
};

// The sequence of jobs every role walks through in the same order.  A CTA
// works on two tiles at a time (slots 0 and 1), the slots alternating job by
// job so that the tensor core works on one while the epilogue warps drain the
// other; slot 1 runs (n_layers + 1) / 2 layers behind slot 0, so that the long
// head epilogue of one slot overlaps a hidden layer's MMAs of the other.
// Each slot evaluates n_rounds tiles (round r: tile (r * gridDim.x +
// blockIdx.x) * 2 + slot); every CTA runs the same number of rounds, and
// tiles past the last row are evaluated on zero rows and not stored.
struct JobIter {
  int step = -1, slot = 0, layer = 0, round = 0;
  __device__ int tile() const { return (round * (int)gridDim.x + (int)blockIdx.x) * 2 + slot; }
  // advance to the next job; false when the CTA's work is done
  __device__ bool next(const InferParams& p) {
    const int per_tile = p.n_layers + 1;
    const int lag = per_tile / 2;
    while (true) {
      ++step;
      slot = step & 1;
      const int q = (step >> 1) - (slot ? lag : 0);
      if (q < 0) continue;
      round = q / per_tile;
      layer = q - round * per_tile;
      if (round < p.n_rounds) return true;
      if (slot == 1) return false;  // slot 1 finishes last
    }
  }
};

// Input unit u of a tile: row u % 128, features 8 (u / 128) .. + 7 (zero
// beyond n_in and past the last row).
__device__ __forceinline__ void load_unit(const InferParams& p, int tile, int u, float* xin) {
  const int rr = u & 127, kb = u >> 7;
  const long long xr = (long long)tile * 128 + rr;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int c = kb * 8 + j;
    xin[j] = xr < p.n && c < p.n_in ? p.x[xr * p.n_in + c] : 0.0f;
  }
}
__device__ __forceinline__ void store_unit(const InferParams& p, unsigned char* act, int u,
                                           const float* xin) {
  const uint4 v = make_uint4(pptc::bf16x2_from(xin[0], xin[1]), pptc::bf16x2_from(xin[2], xin[3]),
                             pptc::bf16x2_from(xin[4], xin[5]), pptc::bf16x2_from(xin[6], xin[7]));
  *reinterpret_cast<uint4*>(act + pptc::core_offset(u & 127, u >> 7, p.in_pad)) = v;
}
__device__ __forceinline__ void pack_input(const InferParams& p, unsigned char* act, int tile,
                                           int t) {
  for (int u = t; u < 16 * p.in_pad; u += kEpiThreads) {
    float xin[8];
    load_unit(p, tile, u, xin);
    store_unit(p, act, u, xin);
  }
}

// b/2 of columns cb + 2 (lane % 16) and + 1 in FP32 (0 past the layer's
// width; halving is exact): the bias operand of silu_slice, loaded before the
// accumulator wait so that its latency is hidden.
__device__ __forceinline__ float2 bias_pair(const float* __restrict__ b, int cb, int hidden,
                                            int lane) {
  const int c = cb + 2 * (lane & 15);
  return c < hidden ? make_float2(0.5f * __ldg(b + c), 0.5f * __ldg(b + c + 1))
                    : make_float2(0.0f, 0.0f);
}

// Bias + SiLU of one 32-column slice (columns cb .. cb + 31 of this thread's
// row) into the BF16 activations: h = acc + b/2 (the accumulator holds
// z/2 - b/2), silu = h + h tanh(h) in FP32, one rounding to BF16 per
// activation (the rounding point of the training forward pass).  The packed
// BF16 tanh would save no SFU time (it costs two SFU operations per pair) and
// runs about one BF16 unit low below |h| = 8, which the cancellation in
// h (1 + tanh h) turns into a bias on SiLU's negative branch.  bp is this
// lane's bias_pair of the slice; pair k is broadcast from lane k.
// kFull: all 32 columns exist (no bound checks, fully interleavable).
template <bool kFull>
__device__ __forceinline__ void silu_slice(const uint32_t* v, float2 bp, int cb, int hidden,
                                           unsigned char* act, int r) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    if (!kFull && cb + q * 8 >= hidden) break;
    uint32_t o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = q * 8 + 2 * j;
      const float h0 = __uint_as_float(v[i]) + __shfl_sync(0xffffffffu, bp.x, q * 4 + j);
      const float h1 = __uint_as_float(v[i + 1]) + __shfl_sync(0xffffffffu, bp.y, q * 4 + j);
      o[j] = pptc::bf16x2_from(pptc::silu_half(h0), pptc::silu_half(h1));
    }
    *reinterpret_cast<uint4*>(act + pptc::core_offset(r, (cb >> 3) + q, hidden)) =
        make_uint4(o[0], o[1], o[2], o[3]);
  }
}

__device__ __forceinline__ void epi_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kEpiThreads) : "memory");
}

// Barrier over the epilogue warps that also ANDs a flag across them, so that
// all of them take the same branch after a bounded wait.
__device__ __forceinline__ bool epi_all(bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, 1, %2, p;\n\t"
      "selp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kEpiThreads)
      : "memory");
  return r != 0;
}

// Persistent, warp-specialised network evaluation, 256 rows (two tiles of
// 128) in flight per CTA:
//   warp 0      streams weight chunks into a kRingSlots-deep ring (TMA bulk
//               copies, one mbarrier per slot and direction);
//   warp 1      issues the tcgen05 MMAs of a job (one thread) once the slot's
//               activations are ready, releasing each ring slot by commit;
//   warps 2..17 the epilogue: bias + SiLU back into the slot's activations
//               (in place: the MMAs that read them have completed), or the
//               head (expected count exp(min(o, 30)) and softmax PDF), then
//               the slot's next input tile.
// Warp w reads TMEM lanes 32 (w % 4) .. + 31.  Every wait is bounded; a
// timeout sets the error flag and the roles wind down (copies and MMAs in
// flight are waited for, again bounded, before TMEM is released).
__global__ void __launch_bounds__(kInferThreads, 1)
    infer_kernel(const __grid_constant__ InferParams p) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ __align__(8) uint64_t w_full[kRingSlots], w_empty[kRingSlots];
  __shared__ __align__(8) uint64_t acc_full[2], act_ready[2], mma_done;
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;
  unsigned char* ring = smem + p.ring_off;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) pptc::tmem_alloc(&tmem_slot, 2 * p.slot_cols);
  if (threadIdx.x == 32) {
    for (int i = 0; i < kRingSlots; ++i) {
      pptc::mbar_init(&w_full[i], 1);
      pptc::mbar_init(&w_empty[i], 1);  // released by the commit of the chunk's MMAs
    }
    for (int i = 0; i < 2; ++i) {
      pptc::mbar_init(&acc_full[i], 1);
      pptc::mbar_init(&act_ready[i], kEpiThreads);
    }
    pptc::mbar_init(&mma_done, 1);
    abort_flag = 0;
  }
  pptc::fence_before_sync();
  __syncthreads();
  pptc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  bool ok = true;

  if (warp == 0) {
    // ---------------- weight producer
    if (lane == 0) {
      JobIter it;
      bool more = it.next(p);
      uint32_t k = 0;  // chunks of the shared stream seen
      while (more && ok) {
        const int l = it.layer;
        const int K = l == 0 ? p.in_pad : p.hidden;
        const int rows = l == p.n_layers ? p.out_pad : p.hidden;
        for (int j = 0; j * kChunkK < K; ++j, ++k) {
          const uint32_t slot = k % kRingSlots, use = k / kRingSlots;
          if (abort_flag || !pptc::mbar_wait(&w_empty[slot], (use & 1) ^ 1, p.wait_ns)) {
            ok = false;
            break;
          }
          // each CTA fetches its own copy of every chunk (one bulk copy,
          // completing on the slot's full barrier)
          const uint32_t bytes = (uint32_t)rows * chunk_width(K, j) * 2u;
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                           pptc::smem_u32(&w_full[slot])),
                       "r"(bytes)
                       : "memory");
          if (!(p.skip_first_copy && k == 0))
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
                "[%3];" ::"r"(pptc::smem_u32(ring + slot * kSlotBytes)),
                "l"(p.wpack + p.wpack_off[l] + (size_t)j * rows * kChunkK * 2), "r"(bytes),
                "r"(pptc::smem_u32(&w_full[slot]))
                : "memory");
        }
        more = it.next(p);
      }
      if (!ok) abort_flag = 1;
      // every slot is released (its commit has landed) and every copy has
      // landed before shared memory is given up
      for (uint32_t q = k > kRingSlots ? k - kRingSlots : 0; q < k; ++q) {
        pptc::mbar_wait(&w_full[q % kRingSlots], (q / kRingSlots) & 1, p.wait_ns);
        pptc::mbar_wait(&w_empty[q % kRingSlots], (q / kRingSlots) & 1, p.wait_ns);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      // The issue loop is kept short: the tensor core runs a 128x256x16 MMA
      // in ~128 cycles, and this one thread's bookkeeping between MMAs (waits,
      // descriptors, loop control) must fit in that time or the pipe idles.
      JobIter it;
      bool more = it.next(p);
      uint32_t slot = 0, phase = 0;     // ring slot of the next chunk, its fill parity
      uint32_t jobs[2] = {0u, 0u};      // jobs issued per slot
      // descriptor of ring slot 0 holding a full-width chunk; descriptors
      // advance by adding the byte offset / 16 to the start address field
      // (shared addresses < 256 KB: the field never carries)
      const uint64_t b_full = pptc::smem_desc(pptc::smem_u32(ring), 128, (uint32_t)(kChunkK / 8) * 128u);
      const uint32_t idesc_hidden = pptc::idesc_bf16(128, p.hidden);
      const uint32_t idesc_head = pptc::idesc_bf16(128, p.out_pad);
      while (more && ok) {
        const int T = it.slot, l = it.layer;
        const int K = l == 0 ? p.in_pad : p.hidden;
        if (abort_flag || !pptc::mbar_wait(&act_ready[T], jobs[T] & 1, p.wait_ns)) {
          ok = false;
          break;
        }
        pptc::fence_after_sync();
        const uint32_t d = tmem + (uint32_t)T * p.slot_cols;
        const uint64_t a_desc = pptc::smem_desc(pptc::smem_u32(smem + (size_t)T * p.act_bytes), 128,
                                                (uint32_t)(K / 8) * 128u);
        const uint32_t idesc = l == p.n_layers ? idesc_head : idesc_hidden;
        for (int j = 0; j * kChunkK < K; ++j) {
          if (!pptc::mbar_wait(&w_full[slot], phase, p.wait_ns) || abort_flag) {
            ok = false;
            break;
          }
          pptc::fence_after_sync();
          const uint64_t a_j = a_desc + (uint64_t)(j * (kChunkK / 16) * 16);  // + j * 64 cols * 2 B / 16
          const int w = chunk_width(K, j);
          if (w == kChunkK) {
            const uint64_t b = b_full + (uint64_t)(slot * (kSlotBytes / 16));
#pragma unroll
            for (int s = 0; s < kChunkK / 16; ++s)
              pptc::mma_f16(d, a_j + (uint64_t)(s * 16), b + (uint64_t)(s * 16), idesc,
                            j > 0 || s > 0);
          } else {
            const uint64_t b = pptc::smem_desc(pptc::smem_u32(ring + slot * kSlotBytes), 128,
                                               (uint32_t)(w / 8) * 128u);
            for (int s = 0; s < w / 16; ++s)
              pptc::mma_f16(d, a_j + (uint64_t)(s * 16), b + (uint64_t)(s * 16), idesc,
                            j > 0 || s > 0);
          }
          // the slot is free once these MMAs complete
          pptc::mma_commit(&w_empty[slot]);
          if (++slot == kRingSlots) {
            slot = 0;
            phase ^= 1u;
          }
        }
        if (!ok) break;
        pptc::mma_commit(&acc_full[T]);
        jobs[T]++;
        more = it.next(p);
      }
      // everything issued has completed before TMEM and shared memory go away
      pptc::mma_commit(&mma_done);
      if (!pptc::mbar_wait(&mma_done, 0, p.wait_ns)) ok = false;
      if (!ok) abort_flag = 1;
    }
    __syncwarp();
  } else {
    // ---------------- epilogue
    const int t = threadIdx.x - 64;
    const int ew = warp - 2;
    const int quad = warp & 3;  // TMEM lane quarter this warp may access
    const int cgrp = ew >> 2;   // column group 0..3
    const int r = quad * 32 + lane;
    // the head's biases for the one-pass head (visible to every epilogue
    // thread after the first epi_all barrier, long before the first head)
    float* head_bias = reinterpret_cast<float*>(smem + p.head_bias_off);
    if (p.head_bias_off)
      for (int c = t; c < p.out_pad; c += kEpiThreads) head_bias[c] = p.P[p.off_b[p.n_layers] + c];
    // first tiles of both slots
    for (int T = 0; T < 2; ++T) {
      pack_input(p, smem + (size_t)T * p.act_bytes, (int)blockIdx.x * 2 + T, t);
      pptc::fence_async_smem();
      pptc::mbar_arrive(&act_ready[T]);
    }
    JobIter it;
    bool more = it.next(p);
    uint32_t jobs[2] = {0u, 0u};
    while (more) {
      const int T = it.slot, l = it.layer;
      unsigned char* act = smem + (size_t)T * p.act_bytes;
      // this lane's bias values of the job's two column slices, loaded
      // before the wait (the inner loops broadcast them by shuffle): b for
      // the head, pairs of b/2 for a hidden layer
      const bool head = l == p.n_layers;
      const float* __restrict__ bias = p.P + p.off_b[l];
      const int s0 = cgrp * 32, s1 = (cgrp + 4) * 32;
      const float bl0 = head && s0 + lane < p.out_pad ? __ldg(bias + s0 + lane) : 0.0f;
      const float bl1 = head && s1 + lane < p.out_pad ? __ldg(bias + s1 + lane) : 0.0f;
      const float2 bp0 = head ? make_float2(0.0f, 0.0f) : bias_pair(bias, s0, p.hidden, lane);
      const float2 bp1 =
          head ? make_float2(0.0f, 0.0f) : bias_pair(bias, s0 + 128, p.hidden, lane);
      if (!epi_all(pptc::mbar_wait(&acc_full[T], jobs[T] & 1, p.wait_ns))) {
        ok = false;
        break;
      }
      jobs[T]++;
      pptc::fence_after_sync();
      const uint32_t trow = tmem + (uint32_t)T * p.slot_cols + ((uint32_t)(quad * 32) << 16);
      if (l < p.n_layers) {
        // two 32-column slices per load-wait (columns c0 and c0 + 128)
        for (int c0 = cgrp * 32; c0 < p.hidden; c0 += 256) {
          uint32_t v[2][32];
          const bool two = c0 + 128 < p.hidden;
          pptc::tmem_ld32_nowait(trow + (uint32_t)c0, v[0]);
          if (two) pptc::tmem_ld32_nowait(trow + (uint32_t)(c0 + 128), v[1]);
          pptc::tmem_wait();
          // (hidden <= 256: one pass with the preloaded pairs; wider layers
          // load theirs here)
          const float2 b0 = c0 == s0 ? bp0 : bias_pair(bias, c0, p.hidden, lane);
          const float2 b1 = c0 == s0 ? bp1 : bias_pair(bias, c0 + 128, p.hidden, lane);
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (h == 1 && !two) break;
            const int cb = c0 + h * 128;
            const float2 bp = h ? b1 : b0;
            if (cb + 32 <= p.hidden) silu_slice<true>(v[h], bp, cb, p.hidden, act, r);
            else silu_slice<false>(v[h], bp, cb, p.hidden, act, r);
          }
        }
      } else {
        // head: every epilogue warp takes the 32-column slices cgrp and
        // cgrp + 4 of its 32 rows; row maximum and normaliser are combined
        // across the four column groups in shared memory
        const int tile = it.tile();
        const long long row0 = (long long)tile * 128;
        const long long row = row0 + r;
        const int ld = p.n_bins + 1;  // odd stride: the 32 rows of a warp hit 32 banks
        float* stage = reinterpret_cast<float*>(act);
        // row max / sum per column group, at the end of the slot's buffer
        float(*s_max)[128] = reinterpret_cast<float(*)[128]>(act + p.act_bytes - kRedBytes);
        float(*s_sum)[128] = s_max + 4;
        // the slot's next input, loaded now so that its latency overlaps the head
        const int next = tile + 2 * (int)gridDim.x;
        const int units = 16 * p.in_pad;  // 128 rows x in_pad / 8 chunks of 8
        // one-pass head (PDF output requested and the layout allows it)
        const bool one_pass = p.head_bias_off != 0 && p.pdf != nullptr;
        const bool prefetch = units <= kEpiThreads && !one_pass;
        float xin[8];
        const bool more_rounds = it.round + 1 < p.n_rounds;
        if (prefetch && t < units && more_rounds) load_unit(p, next, t, xin);
        if (one_pass) {
          // one pass: this warp's 32-column slice (if any) is read once; each
          // 16-column half's exponentials go to the staging rows relative to
          // the half's own maximum, the halves' (max, sum) partials meet in
          // shared memory, and the copy-out applies each half's scale
          constexpr float kLog2e = 1.44269504f;
          float(*h_max)[128] = reinterpret_cast<float(*)[128]>(act + p.act_bytes - kHeadRedBytes);
          float(*h_sum)[128] = h_max + 8;
          float* h_scale = reinterpret_cast<float*>(h_sum + 8);  // [128][8]
          float o0 = 0.0f;
          float mh[2] = {-INFINITY, -INFINITY}, sh[2] = {0.0f, 0.0f};
          const int cb = cgrp * 32;
          if (cb < p.out_pad) {
            uint32_t e[32];  // columns cb .. cb + 31 (within the slot's accumulator)
            pptc::tmem_ld32_nowait(trow + (uint32_t)cb, e);
            pptc::tmem_wait();
            const float4* hb = reinterpret_cast<const float4*>(head_bias + cb);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              if (cb + 4 * q < p.out_pad) {  // the bias table holds out_pad values
                const float4 b = hb[q];
                e[4 * q] = __float_as_uint(__uint_as_float(e[4 * q]) + b.x);
                e[4 * q + 1] = __float_as_uint(__uint_as_float(e[4 * q + 1]) + b.y);
                e[4 * q + 2] = __float_as_uint(__uint_as_float(e[4 * q + 2]) + b.z);
                e[4 * q + 3] = __float_as_uint(__uint_as_float(e[4 * q + 3]) + b.w);
              }
            }
            if (cb == 0) o0 = __uint_as_float(e[0]);
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              float m = -INFINITY, se = 0.0f;
#pragma unroll
              for (int i = 16 * hh; i < 16 * hh + 16; ++i) {
                const int c = cb + i;
                if (c >= 1 && c <= p.n_bins) m = fmaxf(m, __uint_as_float(e[i]));
              }
#pragma unroll
              for (int i = 16 * hh; i < 16 * hh + 16; ++i) {
                const int c = cb + i;
                if (c >= 1 && c <= p.n_bins) {
                  const float x = pptc::ex2_approx((__uint_as_float(e[i]) - m) * kLog2e);
                  se += x;
                  stage[r * ld + c - 1] = x;
                }
              }
              mh[hh] = m;
              sh[hh] = se;
            }
          }
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            h_max[cgrp * 2 + hh][r] = mh[hh];
            h_sum[cgrp * 2 + hh][r] = sh[hh];
          }
          if (cgrp == 0 && row < p.n) p.expect[row] = __expf(fminf(o0, 30.0f));
          epi_sync();
          {
            float M = -INFINITY;
#pragma unroll
            for (int w = 0; w < 8; ++w) M = fmaxf(M, h_max[w][r]);
            float S = 0.0f;
#pragma unroll
            for (int w = 0; w < 8; ++w) {
              const float mw = h_max[w][r];
              S += mw == -INFINITY ? 0.0f : h_sum[w][r] * pptc::ex2_approx((mw - M) * kLog2e);
            }
            // this warp's two halves: scale = 2^((m_h - M) log2 e) / S
#pragma unroll
            for (int hh = 0; hh < 2; ++hh) {
              const float mh = h_max[cgrp * 2 + hh][r];
              h_scale[r * 8 + cgrp * 2 + hh] =
                  mh == -INFINITY ? 0.0f : __fdividef(pptc::ex2_approx((mh - M) * kLog2e), S);
            }
          }
          epi_sync();
          const long long left = p.n - row0;
          const int nrows = left < 128 ? (int)left : 128;
          float* dst = p.pdf + row0 * p.n_bins;
          for (int rr = ew; rr < nrows; rr += kEpiWarps)
            for (int c = lane; c < p.n_bins; c += 32)
              dst[rr * p.n_bins + c] = stage[rr * ld + c] * h_scale[rr * 8 + ((c + 1) >> 4)];
        } else {
        // pass 1: the log count and this warp's part of the row maximum
        float o0 = 0.0f, mx = -INFINITY;
#pragma unroll 1
        for (int sl = cgrp; sl * 32 < p.out_pad; sl += 4) {
          uint32_t v[32];
          pptc::tmem_ld32_nowait(trow + (uint32_t)(sl * 32), v);
          pptc::tmem_wait();
          const float bsl = sl == cgrp ? bl0 : bl1;
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int c = sl * 32 + i;
            const float z = __uint_as_float(v[i]) + __shfl_sync(0xffffffffu, bsl, i);
            if (c == 0) o0 = z;
            else if (c <= p.n_bins) mx = fmaxf(mx, z);
          }
        }
        if (cgrp == 0 && row < p.n) p.expect[row] = __expf(fminf(o0, 30.0f));
        if (p.pdf) {
          s_max[cgrp][r] = mx;
          epi_sync();
          mx = fmaxf(fmaxf(s_max[0][r], s_max[1][r]), fmaxf(s_max[2][r], s_max[3][r]));
          // pass 2: exponentials (into the staging rows, normalised on the way
          // out) and this warp's part of the normaliser
          float se = 0.0f;
#pragma unroll 1
          for (int sl = cgrp; sl * 32 < p.out_pad; sl += 4) {
            uint32_t v[32];
            pptc::tmem_ld32_nowait(trow + (uint32_t)(sl * 32), v);
            pptc::tmem_wait();
            const float bsl = sl == cgrp ? bl0 : bl1;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const int c = sl * 32 + i;
              const float bc = __shfl_sync(0xffffffffu, bsl, i);
              if (c >= 1 && c <= p.n_bins) {
                const float e = __expf(__uint_as_float(v[i]) + bc - mx);
                se += e;
                if (p.stage_pdf) stage[r * ld + c - 1] = e;
              }
            }
          }
          s_sum[cgrp][r] = se;
          epi_sync();
          if (p.stage_pdf) {
            const long long left = p.n - row0;
            const int nrows = left < 128 ? (int)left : 128;
            float* dst = p.pdf + row0 * p.n_bins;
            for (int rr = ew; rr < nrows; rr += kEpiWarps) {
              const float inv =
                  1.0f / (s_sum[0][rr] + s_sum[1][rr] + s_sum[2][rr] + s_sum[3][rr]);
              for (int c = lane; c < p.n_bins; c += 32)
                dst[rr * p.n_bins + c] = stage[rr * ld + c] * inv;
            }
          } else {
            // pass 3 (PDF rows too wide to stage): normalised values straight out
            const float inv = 1.0f / (s_sum[0][r] + s_sum[1][r] + s_sum[2][r] + s_sum[3][r]);
#pragma unroll 1
            for (int sl = cgrp; sl * 32 < p.out_pad; sl += 4) {
              uint32_t v[32];
              pptc::tmem_ld32_nowait(trow + (uint32_t)(sl * 32), v);
              pptc::tmem_wait();
              const float bsl = sl == cgrp ? bl0 : bl1;
#pragma unroll
              for (int i = 0; i < 32; ++i) {
                const int c = sl * 32 + i;
                const float bc = __shfl_sync(0xffffffffu, bsl, i);
                if (c >= 1 && c <= p.n_bins && row < p.n)
                  p.pdf[row * p.n_bins + c - 1] = __expf(__uint_as_float(v[i]) + bc - mx) * inv;
              }
            }
          }
        }
        }  // multi-pass head
        epi_sync();  // the slot's buffer is read out before the next input lands
        if (more_rounds) {
          if (prefetch) {
            if (t < units) store_unit(p, act, t, xin);
          } else {
            pack_input(p, act, next, t);
          }
        }
      }
      pptc::fence_async_smem();  // activation writes -> the next MMAs of this slot
      pptc::fence_before_sync();
      pptc::mbar_arrive(&act_ready[T]);
      more = it.next(p);
    }
    if (!ok) abort_flag = 1;
  }
  pptc::fence_before_sync();
  __syncthreads();
  if (warp == 0) pptc::tmem_dealloc(tmem, 2 * p.slot_cols);
  if (threadIdx.x == 0 && (abort_flag || !ok)) atomicOr(p.err, 1u);
}

int fail(int code, const std::string& m) { return pp::report_error(code, m); }
int cuda_fail(cudaError_t e, const char* what) {
  return fail(PP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Grid: 128-row tiles x 128-column tiles x K splits of at most 256.  The
// split size must be a multiple of kKC (except when one split covers all of K).
// The GEMM's shared-memory opt-in, once per process (before any capture).
cudaError_t gemm_setup() {
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(kGemmStages * kStageBytes));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  return cudaSuccess;
}

// Launch with programmatic stream serialisation (the kernel begins with
// pdl_begin).
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                       cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

cudaError_t launch_gemm(const GemmParams& p, cudaStream_t s) {
  if (cudaError_t e = gemm_setup()) return e;
  const int splits = (p.K + p.k_per_split - 1) / p.k_per_split;
  const int stages = std::min(kGemmStages, (p.k_per_split + kKC - 1) / kKC);
  dim3 grid((p.M + kTileM - 1) / kTileM, (p.N + kTileN - 1) / kTileN, splits);
  return launch_pdl(gemm_kernel, grid, dim3(kGemmThreads), stages * kStageBytes, s, p);
}

inline int pad16(int x) { return (x + 15) & ~15; }
inline long long pad8ll(long long x) { return (x + 7) & ~7LL; }

}  // namespace

// ---------------------------------------------------------------------------
// The network object.
struct pp_mlp {
  int device = 0;
  int n_in = 8, in_pad = 16, hidden = 256, n_layers = 4, n_out = 65, out_pad = 80, n_bins = 64;
  int max_batch = 0;
  long long n_params = 0;
  std::vector<long long> off_w, off_b;  // per layer (n_layers hidden + head)
  std::vector<int> rows, cols;          // W_l is rows x cols (out_pad x in_pad)
  float *P = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;
  bf16* P16 = nullptr;
  bf16* X0 = nullptr;
  std::vector<bf16*> Z, Y;
  float* O = nullptr;
  bf16* dO16 = nullptr;
  bf16* dZ[2] = {nullptr, nullptr};
  float* loss = nullptr;
  unsigned* err = nullptr;
  unsigned char* wpack = nullptr;       // BF16 weights in core-matrix layout
  std::vector<long long> wpack_off;     // bytes per layer
  bool pack_dirty = true;
  int num_sms = 0;
  int infer_ctas = 0;      // co-resident CTAs of the inference kernel
  size_t infer_smem = 0;
  long long step = 0;
  float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f, time_weight = 1.0f;
  // pp_mlp_train_steps: batch buffers, device step counter and schedule
  // scalars, and the captured step with the arguments it was captured for
  float *bx = nullptr, *bc = nullptr, *bh = nullptr;
  long long* d_step = nullptr;
  float* d_sched = nullptr;
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t step_graph = nullptr;
  struct GraphKey {
    const float *x, *c, *h;
    long long n_rows, step0, total;
    int B;
    float lr0, lr1;
    unsigned long long seed;
    bool operator==(const GraphKey& o) const {
      return x == o.x && c == o.c && h == o.h && n_rows == o.n_rows && step0 == o.step0 &&
             total == o.total && B == o.B && lr0 == o.lr0 && lr1 == o.lr1 && seed == o.seed;
    }
  } graph_key{};
};

namespace {

void mlp_free(pp_mlp* m) {
  cudaFree(m->P); cudaFree(m->G); cudaFree(m->Mo); cudaFree(m->Vo); cudaFree(m->P16);
  cudaFree(m->X0); cudaFree(m->O); cudaFree(m->dO16);
  cudaFree(m->dZ[0]); cudaFree(m->dZ[1]); cudaFree(m->loss); cudaFree(m->err);
  cudaFree(m->wpack);
  cudaFree(m->bx); cudaFree(m->bc); cudaFree(m->bh); cudaFree(m->d_step); cudaFree(m->d_sched);
  if (m->step_graph) cudaGraphExecDestroy(m->step_graph);
  if (m->cap_stream) cudaStreamDestroy(m->cap_stream);
  for (auto* p : m->Z) cudaFree(p);
  for (auto* p : m->Y) cudaFree(p);
}

GemmParams base_params(pp_mlp* m) {
  GemmParams p{};
  p.err = m->err;
  return p;
}

int mlp_forward(pp_mlp* m, const float* d_x, int B, cudaStream_t s) {
  const long long nin = (long long)B * m->in_pad;
  cudaError_t e0 = launch_pdl(pack_input_kernel, dim3((unsigned)((nin + 255) / 256)), dim3(256), 0,
                              s, d_x, B, m->n_in, m->in_pad, m->X0);
  if (e0 != cudaSuccess) return cuda_fail(e0, "pack input");
  const bf16* x = m->X0;
  long long ldx = m->in_pad;
  int kin = m->in_pad;
  for (int l = 0; l < m->n_layers; ++l) {
    GemmParams p = base_params(m);
    p.A = x; p.lda = ldx; p.a_trans = 0;
    p.B = m->P16 + m->off_w[l]; p.ldb = m->cols[l]; p.b_trans = 0;
    p.M = B; p.N = m->hidden; p.K = kin; p.k_per_split = kin;
    p.mode = kHiddenFwd; p.bias = m->P + m->off_b[l];
    p.Z16 = m->Z[l]; p.ldz = m->hidden; p.C16 = m->Y[l]; p.ldc16 = m->hidden;
    cudaError_t e = launch_gemm(p, s);
    if (e != cudaSuccess) return cuda_fail(e, "mlp forward gemm");
    x = m->Y[l]; ldx = m->hidden; kin = m->hidden;
  }
  GemmParams p = base_params(m);
  const int L = m->n_layers;
  p.A = x; p.lda = ldx; p.a_trans = 0;
  p.B = m->P16 + m->off_w[L]; p.ldb = m->cols[L]; p.b_trans = 0;
  p.M = B; p.N = m->out_pad; p.K = kin; p.k_per_split = kin;
  p.mode = kStoreF32; p.bias = m->P + m->off_b[L]; p.C32 = m->O; p.ldc = m->out_pad;
  cudaError_t e = launch_gemm(p, s);
  if (e != cudaSuccess) return cuda_fail(e, "mlp head gemm");
  return PP_OK;
}

int mlp_backward(pp_mlp* m, const float* d_count, const float* d_hist, int B, cudaStream_t s) {
  cudaError_t e = launch_pdl(zero_kernel, dim3((unsigned)((m->n_params + 255) / 256)), dim3(256),
                             0, s, m->G, m->n_params, m->loss);
  if (e != cudaSuccess) return cuda_fail(e, "zero gradients");
  const int L = m->n_layers;
  e = launch_pdl(loss_kernel, dim3((unsigned)std::min(256, (B + kLossWarps - 1) / kLossWarps)),
                 dim3(kLossWarps * 32), 0, s, (const float*)m->O, (long long)m->out_pad, B,
                 d_count, d_hist, m->n_bins, 1.0f / (float)B, m->time_weight, m->dO16,
                 (long long)m->out_pad, m->out_pad, m->G + m->off_b[L], m->loss);
  if (e != cudaSuccess) return cuda_fail(e, "loss");
  const int ksplit = kGemmStages * kKC;
  auto colsum16 = [&](const bf16* X, int cols, long long ld, float* out) {
    const unsigned g = (unsigned)std::min(128, (B + kColsumWarps - 1) / kColsumWarps);
    return launch_pdl(colsum_kernel, dim3(g), dim3(kColsumWarps * 32), 0, s, X, B, cols, ld, out);
  };
  // head
  {
    GemmParams p = base_params(m);  // dW_head[o][i] += sum_b dO[b][o] Y[b][i]
    p.A = m->dO16; p.lda = m->out_pad; p.a_trans = 1;
    p.B = m->Y[L - 1]; p.ldb = m->hidden; p.b_trans = 1;
    p.M = m->out_pad; p.N = m->hidden; p.K = B; p.k_per_split = ksplit;
    p.mode = kAccumulateF32; p.C32 = m->G + m->off_w[L]; p.ldc = m->cols[L];
    if ((e = launch_gemm(p, s)) != cudaSuccess) return cuda_fail(e, "dW head");
    GemmParams q = base_params(m);  // dZ[L-1] = (dO W_head) * silu'(Z[L-1])
    q.A = m->dO16; q.lda = m->out_pad; q.a_trans = 0;
    q.B = m->P16 + m->off_w[L]; q.ldb = m->cols[L]; q.b_trans = 1;
    q.M = B; q.N = m->hidden; q.K = m->out_pad; q.k_per_split = m->out_pad;
    q.mode = kBackwardDx; q.Zprev = m->Z[L - 1]; q.ldzp = m->hidden;
    q.C16 = m->dZ[0]; q.ldc16 = m->hidden;
    if ((e = launch_gemm(q, s)) != cudaSuccess) return cuda_fail(e, "dX head");
  }
  int cur = 0;
  for (int l = L - 1; l >= 0; --l) {
    const bf16* xin = l > 0 ? m->Y[l - 1] : m->X0;
    const long long ldx = l > 0 ? m->hidden : m->in_pad;
    const int nin = l > 0 ? m->hidden : m->in_pad;
    if ((e = colsum16(m->dZ[cur], m->hidden, m->hidden, m->G + m->off_b[l])) != cudaSuccess)
      return cuda_fail(e, "bias gradients");
    GemmParams p = base_params(m);  // dW_l[o][i] += sum_b dZ[b][o] x[b][i]
    p.A = m->dZ[cur]; p.lda = m->hidden; p.a_trans = 1;
    p.B = xin; p.ldb = ldx; p.b_trans = 1;
    p.M = m->hidden; p.N = nin; p.K = B; p.k_per_split = ksplit;
    p.mode = kAccumulateF32; p.C32 = m->G + m->off_w[l]; p.ldc = m->cols[l];
    if ((e = launch_gemm(p, s)) != cudaSuccess) return cuda_fail(e, "dW hidden");
    if (l == 0) break;
    GemmParams q = base_params(m);  // dZ[l-1] = (dZ_l W_l) * silu'(Z[l-1])
    q.A = m->dZ[cur]; q.lda = m->hidden; q.a_trans = 0;
    q.B = m->P16 + m->off_w[l]; q.ldb = m->cols[l]; q.b_trans = 1;
    q.M = B; q.N = m->hidden; q.K = m->hidden; q.k_per_split = m->hidden;
    q.mode = kBackwardDx; q.Zprev = m->Z[l - 1]; q.ldzp = m->hidden;
    q.C16 = m->dZ[cur ^ 1]; q.ldc16 = m->hidden;
    if ((e = launch_gemm(q, s)) != cudaSuccess) return cuda_fail(e, "dX hidden");
    cur ^= 1;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mlp backward");
  return PP_OK;
}

int mlp_repack(pp_mlp* m, cudaStream_t s) {
  for (int l = 0; l <= m->n_layers; ++l) {
    const long long n = (long long)m->rows[l] * m->cols[l];
    const bool hidden = l < m->n_layers;
    repack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
        m->P + m->off_w[l], m->rows[l], m->cols[l], hidden ? 0.5f : 1.0f,
        m->wpack + m->wpack_off[l]);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "repack weights");
  m->pack_dirty = false;
  return PP_OK;
}

// Shared memory of infer_kernel: the activations of two tiles (128 rows x
// max(in_pad, hidden) BF16 each, at least the head's reduction arrays), then
// the weight ring.  The head stages a tile's PDF rows (128 x (n_bins + 1)
// floats) in that tile's activation buffer when they fit before the
// reduction arrays at its end.
struct InferSmem {
  uint32_t act, ring_off, total;
  bool stage_pdf;
  uint32_t head_bias_off;  // 0: the multi-pass head
};
InferSmem infer_smem(const pp_mlp* m) {
  const size_t act = std::max<size_t>((size_t)128 * std::max(m->hidden, m->in_pad) * 2, kRedBytes);
  const size_t ring_off = 2 * act;
  const size_t end = ring_off + (size_t)kRingSlots * kSlotBytes;
  const bool stage = (size_t)128 * (m->n_bins + 1) * 4 + kRedBytes <= act;
  // one-pass head: at most one 32-column slice per epilogue warp, PDF rows
  // staged, and room for the head's biases after the ring
  const bool one_pass = (size_t)128 * (m->n_bins + 1) * 4 + kHeadRedBytes <= act &&
                        m->out_pad <= 128 && end + (size_t)m->out_pad * 4 <= (size_t)kMaxInferSmem;
  return {(uint32_t)act, (uint32_t)ring_off,
          (uint32_t)(one_pass ? end + (size_t)m->out_pad * 4 : end), stage,
          one_pass ? (uint32_t)end : 0u};
}

int check_err(pp_mlp* m, cudaStream_t s) {
  unsigned h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, m->err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "mlp");
  if (h) {
    cudaMemsetAsync(m->err, 0, sizeof(unsigned), s);
    return fail(PP_ERR_TIMEOUT, "a tensor-core wait timed out");
  }
  return PP_OK;
}

}  // namespace

extern "C" {

PP_API int pp_mlp_create(pp_mlp** out, int32_t device, int32_t n_in, int32_t hidden,
                         int32_t n_layers, int32_t n_bins, int32_t max_batch, uint64_t seed) {
  if (!out) return fail(PP_ERR_INVALID, "null output");
  *out = nullptr;
  if (n_in < 1 || n_in > 240 || hidden < 16 || hidden > 256 || hidden % 16 || n_layers < 1 ||
      n_layers > 16 || n_bins < 1 || n_bins + 1 > 256 || max_batch < 1)
    return fail(PP_ERR_INVALID, "mlp dims: 1<=n_in<=240, hidden multiple of 16 <= 256, "
                                "n_bins <= 255, max_batch >= 1");
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(PP_ERR_NO_DEVICE, "no CUDA device available");
  }
  cudaSetDevice(device);
  pp_mlp* m = new pp_mlp();
  m->device = device;
  m->n_in = n_in;
  m->in_pad = pad16(n_in);
  m->hidden = hidden;
  m->n_layers = n_layers;
  m->n_bins = n_bins;
  m->n_out = n_bins + 1;
  m->out_pad = pad16(m->n_out);
  m->max_batch = max_batch;
  long long off = 0;
  for (int l = 0; l <= n_layers; ++l) {
    const int r = l < n_layers ? hidden : m->out_pad;
    const int c = l == 0 ? m->in_pad : hidden;
    m->rows.push_back(r);
    m->cols.push_back(c);
    m->off_w.push_back(off);
    off = pad8ll(off + (long long)r * c);
    m->off_b.push_back(off);
    off = pad8ll(off + r);
  }
  m->n_params = off;
  // He-style initialisation of the real (unpadded) weights; zeros elsewhere.
  std::vector<float> h(off, 0.0f);
  uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
  auto rnd = [&]() {  // xorshift64*, uniform (-1, 1)
    st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
    return (double)((st * 2685821657736338717ull) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  };
  for (int l = 0; l <= n_layers; ++l) {
    const int fan_in = l == 0 ? n_in : hidden;
    const int rows_real = l < n_layers ? hidden : m->n_out;
    const double a = std::sqrt(6.0 / fan_in) * (l < n_layers ? 1.0 : 0.1);
    for (int r = 0; r < rows_real; ++r)
      for (int c = 0; c < fan_in; ++c) h[m->off_w[l] + (long long)r * m->cols[l] + c] = (float)(a * rnd());
  }
  const size_t pb = sizeof(float) * off;
  const long long Bn = max_batch;
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
  };
  A((void**)&m->P, pb); A((void**)&m->G, pb); A((void**)&m->Mo, pb); A((void**)&m->Vo, pb);
  A((void**)&m->P16, sizeof(bf16) * off);
  A((void**)&m->X0, sizeof(bf16) * Bn * m->in_pad);
  m->Z.assign(n_layers, nullptr);
  m->Y.assign(n_layers, nullptr);
  for (int l = 0; l < n_layers; ++l) {
    A((void**)&m->Z[l], sizeof(bf16) * Bn * hidden);
    A((void**)&m->Y[l], sizeof(bf16) * Bn * hidden);
  }
  A((void**)&m->O, sizeof(float) * Bn * m->out_pad);
  A((void**)&m->dO16, sizeof(bf16) * Bn * m->out_pad);
  A((void**)&m->dZ[0], sizeof(bf16) * Bn * hidden);
  A((void**)&m->dZ[1], sizeof(bf16) * Bn * hidden);
  A((void**)&m->loss, sizeof(float));
  A((void**)&m->err, sizeof(unsigned));
  long long wbytes = 0;
  for (int l = 0; l <= n_layers; ++l) {
    m->wpack_off.push_back(wbytes);
    wbytes += (long long)m->rows[l] * m->cols[l] * 2;  // rows, cols multiples of 16: 512-byte steps
  }
  A((void**)&m->wpack, (size_t)wbytes);
  if (e == cudaSuccess) e = cudaMemcpy(m->P, h.data(), pb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->Mo, 0, pb);
  if (e == cudaSuccess) e = cudaMemset(m->Vo, 0, pb);
  if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(unsigned));
  if (e == cudaSuccess) {
    to_bf16_kernel<<<(unsigned)((off + 255) / 256), 256>>>(m->P, off, m->P16);
    e = cudaDeviceSynchronize();
  }
  if (e != cudaSuccess) {
    mlp_free(m);
    delete m;
    return cuda_fail(e, "pp_mlp_create");
  }
  *out = m;
  return PP_OK;
}

PP_API int pp_mlp_destroy(pp_mlp* m) {
  if (!m) return PP_OK;
  cudaSetDevice(m->device);
  cudaDeviceSynchronize();
  mlp_free(m);
  delete m;
  return PP_OK;
}

PP_API int pp_mlp_num_params(const pp_mlp* m, int64_t* n) {
  if (!m || !n) return fail(PP_ERR_INVALID, "null argument");
  *n = m->n_params;
  return PP_OK;
}

// Offsets (in floats) of W_l and b_l in the packed parameter vector and the
// padded shape of W_l (rows x cols, row-major).
PP_API int pp_mlp_layout(const pp_mlp* m, int32_t layer, int64_t* off_w, int64_t* off_b,
                         int32_t* rows, int32_t* cols) {
  if (!m || layer < 0 || layer > m->n_layers) return fail(PP_ERR_INVALID, "bad layer");
  if (off_w) *off_w = m->off_w[layer];
  if (off_b) *off_b = m->off_b[layer];
  if (rows) *rows = m->rows[layer];
  if (cols) *cols = m->cols[layer];
  return PP_OK;
}

PP_API int pp_mlp_get_params(const pp_mlp* m, float* host, int64_t n) {
  if (!m || !host || n != m->n_params) return fail(PP_ERR_INVALID, "bad parameter buffer");
  cudaSetDevice(m->device);
  cudaError_t e = cudaMemcpy(host, m->P, sizeof(float) * n, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? PP_OK : cuda_fail(e, "pp_mlp_get_params");
}

PP_API int pp_mlp_set_params(pp_mlp* m, const float* host, int64_t n) {
  if (!m || !host || n != m->n_params) return fail(PP_ERR_INVALID, "bad parameter buffer");
  cudaSetDevice(m->device);
  cudaError_t e = cudaMemcpy(m->P, host, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    to_bf16_kernel<<<(unsigned)((n + 255) / 256), 256>>>(m->P, n, m->P16);
    e = cudaDeviceSynchronize();
  }
  m->pack_dirty = true;
  return e == cudaSuccess ? PP_OK : cuda_fail(e, "pp_mlp_set_params");
}

// Forward pass of the training graph: raw head outputs (B x out_pad, FP32,
// column 0 = log expected count, 1..n_bins = time logits) into d_out.
PP_API int pp_mlp_forward(pp_mlp* m, const float* d_x, int32_t B, float* d_out, void* stream) {
  if (!m || !d_x || !d_out || B < 1 || B > m->max_batch) return fail(PP_ERR_INVALID, "bad arguments");
  cudaSetDevice(m->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = mlp_forward(m, d_x, B, s);
  if (rc != PP_OK) return rc;
  cudaError_t e = cudaMemcpyAsync(d_out, m->O, sizeof(float) * (size_t)B * m->out_pad,
                                  cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy head outputs");
  return check_err(m, s);
}

// Loss and gradient (no update): gradients of the packed parameters to host.
PP_API int pp_mlp_loss_grad(pp_mlp* m, const float* d_x, const float* d_count,
                            const float* d_hist, int32_t B, float* host_grad, float* host_loss,
                            void* stream) {
  if (!m || !d_x || !d_count || !d_hist || B < 1 || B > m->max_batch)
    return fail(PP_ERR_INVALID, "bad arguments");
  cudaSetDevice(m->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = mlp_forward(m, d_x, B, s);
  if (rc == PP_OK) rc = mlp_backward(m, d_count, d_hist, B, s);
  if (rc != PP_OK) return rc;
  cudaError_t e = cudaSuccess;
  if (host_grad) e = cudaMemcpyAsync(host_grad, m->G, sizeof(float) * m->n_params,
                                     cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && host_loss)
    e = cudaMemcpyAsync(host_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "copy gradients");
  return check_err(m, s);
}

// One Adam step on a batch (forward, backward, update), asynchronous on
// `stream`; the batch loss is left in device memory (pp_mlp_last_loss).
PP_API int pp_mlp_train_step(pp_mlp* m, const float* d_x, const float* d_count,
                             const float* d_hist, int32_t B, float lr, void* stream) {
  if (!m || !d_x || !d_count || !d_hist || B < 1 || B > m->max_batch)
    return fail(PP_ERR_INVALID, "bad arguments");
  cudaSetDevice(m->device);
  cudaStream_t s = (cudaStream_t)stream;
  int rc = mlp_forward(m, d_x, B, s);
  if (rc == PP_OK) rc = mlp_backward(m, d_count, d_hist, B, s);
  if (rc != PP_OK) return rc;
  m->step += 1;
  // bias corrections in double, rounded once: the captured step's
  // schedule_kernel computes the same, so that both paths take equal steps
  // (1 - b2^t cancels, and the float pow of host and device libraries can
  // differ by an ulp, ~2e-5 of bc2 at small t)
  const float bc1 = (float)(1.0 - std::pow((double)m->b1, (double)m->step));
  const float bc2 = (float)(1.0 - std::pow((double)m->b2, (double)m->step));
  cudaError_t ea = launch_pdl(adam_kernel, dim3((unsigned)((m->n_params + 255) / 256)), dim3(256),
                              0, s, m->P, (const float*)m->G, m->Mo, m->Vo, m->n_params, lr,
                              m->b1, m->b2, m->eps, bc1, bc2, m->P16);
  if (ea != cudaSuccess) return cuda_fail(ea, "adam");
  m->pack_dirty = true;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? PP_OK : cuda_fail(e, "adam");
}

// Capture one training step (schedule, batch, forward, backward, Adam, step
// count) on the library's own stream into m->step_graph.
int capture_train_step(pp_mlp* m, const pp_mlp::GraphKey& k) {
  if (m->step_graph) {
    cudaGraphExecDestroy(m->step_graph);
    m->step_graph = nullptr;
  }
  cudaError_t e = cudaSuccess;
  if (!m->cap_stream) e = cudaStreamCreateWithFlags(&m->cap_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess && !m->bx) {
    e = cudaMalloc(&m->bx, sizeof(float) * (size_t)m->max_batch * m->n_in);
    if (e == cudaSuccess) e = cudaMalloc(&m->bc, sizeof(float) * (size_t)m->max_batch);
    if (e == cudaSuccess) e = cudaMalloc(&m->bh, sizeof(float) * (size_t)m->max_batch * m->n_bins);
    if (e == cudaSuccess) e = cudaMalloc(&m->d_step, sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&m->d_sched, sizeof(float) * 4);
  }
  if (e == cudaSuccess) e = gemm_setup();
  if (e != cudaSuccess) return cuda_fail(e, "train-step setup");
  cudaStream_t cs = m->cap_stream;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "begin capture");
  // (the first kernel of a step is launched plainly: it follows the previous
  // graph launch)
  schedule_kernel<<<1, 1, 0, cs>>>(m->d_step, k.step0, k.total, k.lr0, k.lr1, m->b1, m->b2,
                                   m->d_sched);
  int rc = PP_OK;
  e = launch_pdl(gather_kernel, dim3((unsigned)((k.B + 7) / 8)), dim3(256), 0, cs, k.x, k.c, k.h,
                 (long long)k.n_rows, m->n_in, m->n_bins, k.B, (const long long*)m->d_step,
                 (uint32_t)k.seed, (uint32_t)(k.seed >> 32), m->bx, m->bc, m->bh);
  if (e != cudaSuccess) rc = cuda_fail(e, "gather");
  if (rc == PP_OK) rc = mlp_forward(m, m->bx, k.B, cs);
  if (rc == PP_OK) rc = mlp_backward(m, m->bc, m->bh, k.B, cs);
  if (rc == PP_OK) {
    e = launch_pdl(adam_dev_kernel, dim3((unsigned)((m->n_params + 255) / 256)), dim3(256), 0, cs,
                   m->P, (const float*)m->G, m->Mo, m->Vo, m->n_params, (const float*)m->d_sched,
                   m->b1, m->b2, m->eps, m->P16);
    if (e == cudaSuccess) e = launch_pdl(step_kernel, dim3(1), dim3(1), 0, cs, m->d_step);
    if (e != cudaSuccess) rc = cuda_fail(e, "adam step");
  }
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);  // always end the capture
  if (rc != PP_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return rc != PP_OK ? rc : cuda_fail(e, "end capture");
  }
  e = cudaGraphInstantiate(&m->step_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    m->step_graph = nullptr;
    return cuda_fail(e, "instantiate train step");
  }
  m->graph_key = k;
  return PP_OK;
}

// Adam state for checkpoints: first and second moments (n floats each, either
// may be null) and the step count.
PP_API int pp_mlp_train_steps(pp_mlp* m, const float* d_x, const float* d_count,
                              const float* d_hist, int64_t n_rows, int32_t B, int32_t n_steps,
                              int64_t step0, int64_t total, float lr0, float lr1, uint64_t seed,
                              void* stream) {
  if (!m || !d_x || !d_count || !d_hist || n_rows < 1 || B < 1 || B > m->max_batch ||
      n_steps < 0 || total < 1 || step0 < 0 || !(lr0 >= 0.0f) || !(lr1 >= 0.0f))
    return fail(PP_ERR_INVALID, "pp_mlp_train_steps: bad arguments");
  if (n_steps == 0) return PP_OK;
  cudaSetDevice(m->device);
  const pp_mlp::GraphKey k{d_x, d_count, d_hist, (long long)n_rows, (long long)step0,
                           (long long)total, (int)B, lr0, lr1, (unsigned long long)seed};
  if (!m->step_graph || !(m->graph_key == k)) {
    const int rc = capture_train_step(m, k);
    if (rc != PP_OK) return rc;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the device counter continues from the host's count
  set_step_kernel<<<1, 1, 0, s>>>(m->d_step, m->step);
  cudaError_t e = cudaGetLastError();
  for (int i = 0; e == cudaSuccess && i < n_steps; ++i) e = cudaGraphLaunch(m->step_graph, s);
  if (e != cudaSuccess) return cuda_fail(e, "pp_mlp_train_steps");
  m->step += n_steps;
  m->pack_dirty = true;
  return PP_OK;
}

PP_API int pp_mlp_step_count(const pp_mlp* m, int64_t* steps) {
  if (!m || !steps) return fail(PP_ERR_INVALID, "null argument");
  *steps = m->step;
  return PP_OK;
}

PP_API int pp_mlp_get_adam(const pp_mlp* m, float* host_m, float* host_v, int64_t n,
                           int64_t* step) {
  if (!m || n != m->n_params) return fail(PP_ERR_INVALID, "bad moment buffers");
  cudaSetDevice(m->device);
  cudaError_t e = cudaSuccess;
  if (host_m) e = cudaMemcpy(host_m, m->Mo, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_v)
    e = cudaMemcpy(host_v, m->Vo, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (step) *step = m->step;
  return e == cudaSuccess ? PP_OK : cuda_fail(e, "pp_mlp_get_adam");
}

PP_API int pp_mlp_set_adam(pp_mlp* m, const float* host_m, const float* host_v, int64_t n,
                           int64_t step) {
  if (!m || !host_m || !host_v || n != m->n_params || step < 0)
    return fail(PP_ERR_INVALID, "bad moment buffers");
  cudaSetDevice(m->device);
  cudaError_t e = cudaMemcpy(m->Mo, host_m, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->Vo, host_v, sizeof(float) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "pp_mlp_set_adam");
  m->step = step;
  return PP_OK;
}

// Fused inference: expected count (exp of the clamped log-count output) and
// the softmax time PDF of n feature rows, one CTA per 128 rows; n is not
// limited by max_batch.  d_pdf may be null.
static int infer_impl(pp_mlp* m, const float* d_x, int64_t n, float* d_expect, float* d_pdf,
                      void* stream, unsigned long long wait_ns, int skip_first_copy) {
  if (!m || !d_x || !d_expect || n < 0) return fail(PP_ERR_INVALID, "bad arguments");
  if (m->n_layers + 1 > kMaxLayers) return fail(PP_ERR_INVALID, "too many layers");
  if (n == 0) return PP_OK;
  if ((n + 127) / 128 > 0x3FFFFFFFLL) return fail(PP_ERR_INVALID, "n too large");
  cudaSetDevice(m->device);
  cudaStream_t s = (cudaStream_t)stream;
  if (m->pack_dirty) {
    int rc = mlp_repack(m, s);
    if (rc != PP_OK) return rc;
  }
  const InferSmem sm = infer_smem(m);
  const size_t smem = sm.total;
  cudaError_t e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "infer smem");
  InferParams p{};
  p.x = d_x; p.n = n; p.n_in = m->n_in; p.in_pad = m->in_pad; p.hidden = m->hidden;
  p.n_layers = m->n_layers; p.out_pad = m->out_pad; p.n_bins = m->n_bins;
  const long long tiles = (n + 127) / 128;
  p.n_tiles = (int)tiles;
  p.slot_cols = 32;
  while (p.slot_cols < (uint32_t)std::max(m->hidden, m->out_pad)) p.slot_cols *= 2;
  p.act_bytes = sm.act; p.ring_off = sm.ring_off; p.head_bias_off = sm.head_bias_off;
  p.stage_pdf = sm.stage_pdf ? 1 : 0;
  p.wpack = m->wpack; p.P = m->P;
  for (int l = 0; l <= m->n_layers; ++l) {
    p.wpack_off[l] = m->wpack_off[l];
    p.off_b[l] = m->off_b[l];
  }
  p.expect = d_expect; p.pdf = d_pdf; p.err = m->err;
  p.wait_ns = wait_ns; p.skip_first_copy = skip_first_copy;
  if (m->num_sms == 0) {
    e = cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device);
    if (e != cudaSuccess) return cuda_fail(e, "SM count");
  }
  if (m->infer_ctas == 0 || m->infer_smem != smem) {
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, infer_kernel, kInferThreads, smem);
    if (e != cudaSuccess) return cuda_fail(e, "inference occupancy");
    if (per_sm < 1) return fail(PP_ERR_CUDA, "inference kernel: no CTA fits an SM");
    m->infer_ctas = per_sm * m->num_sms;
    m->infer_smem = smem;
  }
  // co-resident CTAs, each with two tiles per round
  const long long grid = std::min<long long>(m->infer_ctas, (tiles + 1) / 2);
  p.n_rounds = (int)((tiles + 2 * grid - 1) / (2 * grid));
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(kInferThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cfg.gridDim = dim3((unsigned)grid);
  e = cudaLaunchKernelEx(&cfg, infer_kernel, p);
  if (e != cudaSuccess) return cuda_fail(e, "infer kernel");
  e = cudaGetLastError();
  return e == cudaSuccess ? PP_OK : cuda_fail(e, "infer kernel");
}

PP_API int pp_mlp_infer(pp_mlp* m, const float* d_x, int64_t n, float* d_expect, float* d_pdf,
                        void* stream) {
  return infer_impl(m, d_x, n, d_expect, d_pdf, stream, kWaitNs, 0);
}

PP_API int pp_mlp_debug_infer_timeout(pp_mlp* m, const float* d_x, int64_t n, float* d_expect,
                                      int64_t wait_ns, void* stream) {
  if (!m || !d_x || !d_expect || n < 1) return fail(PP_ERR_INVALID, "bad arguments");
  if (wait_ns < 1000 || wait_ns > 2000000000)
    return fail(PP_ERR_INVALID, "wait_ns must be in [1e3, 2e9]");
  int rc = infer_impl(m, d_x, n, d_expect, nullptr, stream, (unsigned long long)wait_ns, 1);
  if (rc != PP_OK) return rc;
  return check_err(m, (cudaStream_t)stream);
}

// Device error flag of the tensor-core kernels (timeouts), checked and cleared.
PP_API int pp_mlp_check(pp_mlp* m, void* stream) {
  if (!m) return fail(PP_ERR_INVALID, "null argument");
  cudaSetDevice(m->device);
  return check_err(m, (cudaStream_t)stream);
}

PP_API int pp_mlp_last_loss(pp_mlp* m, float* host_loss) {
  if (!m || !host_loss) return fail(PP_ERR_INVALID, "null argument");
  cudaSetDevice(m->device);
  cudaError_t e = cudaMemcpy(host_loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read loss");
  return check_err(m, nullptr);
}

// One tcgen05 GEMM for tests: C (M x N, FP32) = A (M x K) * B^T with B given
// as N x K (both BF16, row-major, device memory); N <= 256, N and K multiples
// of 16, lda/ldb multiples of 8.
PP_API int pp_mlp_gemm_test(const void* d_a, int64_t lda, int32_t a_trans, const void* d_b,
                            int64_t ldb, int32_t b_trans, int32_t M, int32_t N, int32_t K,
                            int32_t k_split, float* d_c, int64_t ldc, void* stream) {
  if (!d_a || !d_b || !d_c || M < 1 || N < 16 || N > 256 || N % 16 || K < 16 || K % 16 ||
      lda % 8 || ldb % 8)
    return fail(PP_ERR_INVALID, "bad gemm arguments");
  unsigned* err = nullptr;
  cudaError_t e = cudaMalloc(&err, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(err, 0, sizeof(unsigned));
  if (e != cudaSuccess) return cuda_fail(e, "gemm test");
  GemmParams p{};
  p.A = (const bf16*)d_a; p.lda = lda; p.a_trans = a_trans;
  p.B = (const bf16*)d_b; p.ldb = ldb; p.b_trans = b_trans;
  p.M = M; p.N = N; p.K = K;
  p.k_per_split = k_split > 0 ? ((K + k_split - 1) / k_split + kKC - 1) / kKC * kKC : K;
  if (p.k_per_split > kGemmStages * kKC) {
    cudaFree(err);
    return fail(PP_ERR_INVALID, "gemm test: at most 256 of K per split");
  }
  p.mode = k_split > 0 ? kAccumulateF32 : kStoreF32;
  p.C32 = d_c; p.ldc = ldc; p.err = err;
  e = launch_gemm(p, (cudaStream_t)stream);
  unsigned h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) return cuda_fail(e, "gemm test");
  return h ? fail(PP_ERR_TIMEOUT, "tensor-core wait timed out") : PP_OK;
}

}  // extern "C"
