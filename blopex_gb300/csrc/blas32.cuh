// blas32.cuh -- building blocks of the FP32 column kernels (dot products and
// the inner-CG preconditioner's fused updates): 16-byte vector access and an
// FP32 accumulator that keeps FP64-level accuracy.
//
// On this GPU the FP64 pipe runs at 1/64 of the FP32 rate, so an FP32 dot
// product that accumulates in FP64 is bound by its DFMAs, not by HBM.  Here
// each product a b is made exact as p + e (e = fma(a, b, -p)) and added to a
// compensated FP32 sum (Knuth's two-sum); every 64 terms the pair (s, c) is
// flushed into an FP64 accumulator.  The intrinsics keep the compiler from
// contracting the two-sum into FMAs, which would break its error term.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

static __device__ __forceinline__ void acc_prod32(float& s, float& c, float a, float b)
{
  const float p = __fmul_rn(a, b);
  const float e = fmaf(a, b, -p);  // a b = p + e exactly (no underflow)
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  c = __fadd_rn(c, __fadd_rn(err, e));
  s = t;
}

static __device__ __forceinline__ void acc_prod32x4(float& s, float& c, float4 a, float4 b)
{
  acc_prod32(s, c, a.x, b.x);
  acc_prod32(s, c, a.y, b.y);
  acc_prod32(s, c, a.z, b.z);
  acc_prod32(s, c, a.w, b.w);
}

// block-wide sum of one double per thread (blockDim.x = 256), the result in
// thread 0, in a fixed order
static __device__ __forceinline__ double block_sum256(double v)
{
  __shared__ double red[256];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  return red[0];
}

static inline bool cols_aligned16(const void* const* cols, int w)
{
  for (int j = 0; j < w; j++)
    if ((uintptr_t)cols[j] & 15) return false;
  return true;
}
