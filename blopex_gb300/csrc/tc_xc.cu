// tc_xc.cu -- the block updates Y = X C (+ Z) of the explicit FP32 iteration
// (P = [R P] C_RP, X = X C_X + P and their A-images) on the 5th-generation
// tensor cores; they replace serial_Multi_VectorByMatrix
// (blopex_serial_double/multivector/multi_vector.c:474-524, reached through
// lobpcg.c:1212-1262) for FP32 blocks.  X has h <= 128 columns, Y w <= 64;
// C is the FP64 h x w coordinate block on the device.
//
// Compensated TF32 (hi*hi + hi*lo + lo*hi): the update writes the blocks
// themselves, so its products must carry FP32 accuracy.
//
// Per CTA (one per SM, persistent over 128-row tiles):
//   warps 8-15  copy 32-column x 128-row pieces of X into a raw shared
//               buffer with cp.async (column-major as in HBM, NRAW pieces in
//               flight), then transpose each piece into the 128-byte-swizzled
//               K-major operand layout (rows = the 128 block rows, K = the 32
//               columns) as hi and lo TF32 parts;
//   warp 0      allocates TMEM; one thread issues tcgen05.mma.kind::tf32
//               (M = 128, N = NW) per 8-column step into one of two TMEM
//               accumulators (double-buffered over tiles);
//   warps 4-7   read the accumulator of a finished tile (tcgen05.ld, lane =
//               row), add Z and store Y: a warp writes 32 consecutive rows of
//               a column (128 bytes).
// C is converted once per CTA into the B operand (N = output column, K =
// input column).  Every wait is bounded; a timeout sets an error word.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "tc_common.cuh"

#define TCX_THREADS 512
#define TCX_NPROD 256  // warps 8-15
#define TCX_NSTAGE 2   // swizzled (hi + lo) stages consumed by the MMAs
#define TCX_NRAW 4     // raw cp.async pieces in flight
#define TCX_MAX_H 128
#define TCX_PIECE 16384  // 32 columns x 128 rows x 4 bytes

struct tcx_params {
  blk_cols x, y, z;
  const double* C;
  int ldc, h, w, has_z;
  long n;
  int* err;
};

template <int NW>
struct tcx_cfg {
  static constexpr int CB = NW * 128;            // one 32-column K block of C, hi or lo
  static constexpr int C_BYTES = 4 * 2 * CB;     // up to 4 K blocks, hi + lo
  static constexpr int STAGE = 2 * TCX_PIECE;    // hi + lo operand tile
  static constexpr int SMEM = C_BYTES + TCX_NSTAGE * STAGE + TCX_NRAW * TCX_PIECE + 1024;
  static constexpr int TMEM_COLS = 2 * NW;
};

// issue the cp.async copies of piece q (tile, 32-column block) into raw slot
__device__ __forceinline__ void tcx_issue(const tcx_params& prm, unsigned char* raw, long q, int KB,
                                          long ntiles_total, int p)
{
  const long i = q / KB;
  const int kb = (int)(q % KB);
  const long tile = blockIdx.x + i * gridDim.x;
  if (tile >= ntiles_total) return;
  const long r0 = tile * 128;
  for (int u = p; u < 32 * 32; u += TCX_NPROD) {  // 32 columns x 32 four-row pieces
    const int col = u >> 5, r4 = u & 31;
    const int c = kb * 32 + col;
    const long r = r0 + 4 * r4;
    long left = (prm.n - r) * 4;
    uint32_t bytes = c < prm.h ? (left >= 16 ? 16u : (left > 0 ? (uint32_t)left : 0u)) : 0u;
    const float* base = (const float*)prm.x.col[c < prm.h ? c : 0];
    cp_async16(smem_u32(raw + col * 512 + r4 * 16), base + (bytes ? r : 0), bytes);
  }
}

template <int NW>
__global__ void __launch_bounds__(TCX_THREADS, 1) tc_xc_kernel(const __grid_constant__ tcx_params prm)
{
  using G = tcx_cfg<NW>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_align1024(smem_raw);
  unsigned char* cmat = smem;                         // [kb][hi, lo][NW rows][128 B]
  unsigned char* stages = smem + G::C_BYTES;          // [s][hi, lo][128 rows][128 B]
  unsigned char* raws = stages + TCX_NSTAGE * G::STAGE;  // [slot][32 cols][128 rows] FP32
  __shared__ uint64_t full_bar[TCX_NSTAGE], empty_bar[TCX_NSTAGE], accf[2], acce[2], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int KB = (prm.h + 31) >> 5;
  const long ntiles = (prm.n + 127) / 128;
  const long my_tiles = (long)blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;
  const long nq = my_tiles * KB;

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < TCX_NSTAGE; s++) {
      mbar_init(&full_bar[s], TCX_NPROD);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 128);
    }
    mbar_init(&done_bar, 1);
  }
  // B operand: row j (output column) holds C[0..h, j] as TF32 hi / lo
  for (int e = tid; e < NW * KB * 32; e += TCX_THREADS) {
    const int j = e % NW, c = e / NW;
    const float v = (j < prm.w && c < prm.h) ? (float)prm.C[c + (size_t)j * prm.ldc] : 0.f;
    float hi, lo;
    tf32_split(v, hi, lo);
    const int kb = c >> 5, cc = c & 31;
    const uint32_t off = j * 128 + ((((cc >> 2) ^ (j & 7))) << 4) + (cc & 3) * 4;
    *(float*)(cmat + kb * 2 * G::CB + off) = hi;
    *(float*)(cmat + kb * 2 * G::CB + G::CB + off) = lo;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"((uint32_t)G::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp >= 8) {
    // ------------------------------------------------------------ producers
    const int p = tid - 256;
    for (int q = 0; q < TCX_NRAW; q++) {
      if (q < nq) tcx_issue(prm, raws + q * TCX_PIECE, q, KB, ntiles, p);
      cp_async_commit();
    }
    for (long q = 0; q < nq; q++) {
      const int s = (int)(q % TCX_NSTAGE);
      unsigned char* raw = raws + (q % TCX_NRAW) * TCX_PIECE;
      cp_async_wait<TCX_NRAW - 1>();
      named_bar(1, TCX_NPROD);  // every producer's copies of piece q have landed
      bool ok = true;
      if (q >= TCX_NSTAGE) ok = mbar_wait(&empty_bar[s], (uint32_t)(((q / TCX_NSTAGE) - 1) & 1), &abort_flag);
      if (!ok) {
        abort_flag = 1;
        atomicExch(prm.err, 1);
      }
      if (!abort_flag) {
        unsigned char* st = stages + s * G::STAGE;
        for (int u = p; u < 128 * 8; u += TCX_NPROD) {  // (row, 4-column group)
          const int row = u & 127, g = u >> 7;
          float4 v;
          v.x = *(const float*)(raw + (4 * g + 0) * 512 + row * 4);
          v.y = *(const float*)(raw + (4 * g + 1) * 512 + row * 4);
          v.z = *(const float*)(raw + (4 * g + 2) * 512 + row * 4);
          v.w = *(const float*)(raw + (4 * g + 3) * 512 + row * 4);
          float4 hi, lo;
          tf32_split(v.x, hi.x, lo.x);
          tf32_split(v.y, hi.y, lo.y);
          tf32_split(v.z, hi.z, lo.z);
          tf32_split(v.w, hi.w, lo.w);
          const uint32_t off = row * 128 + ((g ^ (row & 7)) << 4);
          *(float4*)(st + off) = hi;
          *(float4*)(st + TCX_PIECE + off) = lo;
        }
        fence_proxy_async();
        mbar_arrive(&full_bar[s]);
      }
      named_bar(1, TCX_NPROD);  // raw slot q is free again
      if (!abort_flag && q + TCX_NRAW < nq) tcx_issue(prm, raw, q + TCX_NRAW, KB, ntiles, p);
      cp_async_commit();
    }
    cp_async_wait<0>();
  } else if (warp == 0 && lane == 0) {
    // ----------------------------------------------------------- MMA issuer
    const uint32_t idesc = tf32_idesc(128, NW);
    const uint32_t cbase = smem_u32(cmat), sbase = smem_u32(stages);
    long q = 0;
    for (long i = 0; i < my_tiles && !abort_flag; i++) {
      const int buf = (int)(i & 1);
      if (i >= 2 && !mbar_wait(&acce[buf], (uint32_t)(((i >> 1) - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 2);
        break;
      }
      tc_fence_after();
      const uint32_t d = tmem + (uint32_t)(buf * NW);
      for (int kb = 0; kb < KB; kb++, q++) {
        const int s = (int)(q % TCX_NSTAGE);
        if (!mbar_wait(&full_bar[s], (uint32_t)((q / TCX_NSTAGE) & 1), &abort_flag)) {
          abort_flag = 1;
          atomicExch(prm.err, 3);
          break;
        }
        tc_fence_after();
        const uint32_t a = sbase + s * G::STAGE, b = cbase + kb * 2 * G::CB;
        for (int kk = 0; kk < 4; kk++) {
          const uint32_t acc = (kb > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(d, sw128_desc(a + kk * 32), sw128_desc(b + kk * 32), idesc, acc);
          mma_tf32(d, sw128_desc(a + kk * 32), sw128_desc(b + G::CB + kk * 32), idesc, 1u);
          mma_tf32(d, sw128_desc(a + TCX_PIECE + kk * 32), sw128_desc(b + kk * 32), idesc, 1u);
        }
        mma_commit(&empty_bar[s]);
      }
      if (abort_flag) break;
      mma_commit(&accf[buf]);
    }
    mma_commit(&done_bar);
  } else if (warp >= 4 && warp < 8) {
    // ------------------------------------------------------------- epilogue
    const int quarter = warp - 4;
    for (long i = 0; i < my_tiles; i++) {
      const int buf = (int)(i & 1);
      const long row = (blockIdx.x + i * gridDim.x) * 128 + 32 * quarter + lane;
      // Z does not depend on the products: all of this row's loads are in
      // flight while the tile's MMAs run (and ahead of the Y stores, which
      // the compiler could not reorder across possibly aliasing loads)
      float zv[NW];
#pragma unroll
      for (int j = 0; j < NW; j++)
        zv[j] = (prm.has_z && j < prm.w && row < prm.n) ? ((const float*)prm.z.col[j])[row] : 0.f;
      const bool got = mbar_wait(&accf[buf], (uint32_t)((i >> 1) & 1), &abort_flag);
      if (!__all_sync(0xffffffffu, got)) {  // tcgen05.ld needs the whole warp
        abort_flag = 1;
        atomicExch(prm.err, 4);
        break;
      }
      tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(buf * NW);
#pragma unroll
      for (int g = 0; g < NW / 32; g++) {
        uint32_t r[32];
        tmem_ld32(taddr + g * 32, r);
        if (row < prm.n) {
#pragma unroll
          for (int jj = 0; jj < 32; jj++) {
            const int j = g * 32 + jj;
            if (j < prm.w) ((float*)prm.y.col[j])[row] = __uint_as_float(r[jj]) + zv[j];
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acce[buf]);
    }
  }
  // TMEM is freed only after the last MMA has completed (done_bar is always
  // committed by the issuer) and every epilogue read has finished
  if (warp == 0) {
    mbar_drain(&done_bar, 0);
    __syncwarp();
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)G::TMEM_COLS)
                 : "memory");
  }
}

template <int NW>
static int tcx_launch(gpu_Context* ctx, const tcx_params& prm, int nctas)
{
  const int smem = tcx_cfg<NW>::SMEM;
  if (cudaFuncSetAttribute(tc_xc_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return gb_fail(ctx, "tc_xc: cannot reserve %d bytes of shared memory", smem);
  if (tc_apply_wait_polls(ctx->opt.wait_polls, (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "tc_xc: cannot set the wait limit");
  tc_xc_kernel<NW><<<nctas, TCX_THREADS, smem, (cudaStream_t)ctx->stream>>>(prm);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "tc_xc");
}

__global__ void tcx_check_kernel(const int* err, int* status)
{
  if (*err) *status = *err;
}

extern "C" int gb_tc_xc(gpu_Context* ctx, long n, const blk_cols* X, int h, const double* C, int ldc,
                        const blk_cols* Y, int w, const blk_cols* Z)
{
  if (n <= 0 || w <= 0) return 0;
  if (h < 1 || h > TCX_MAX_H || w > 64)
    return gb_fail(ctx, "tc_xc: block widths (%d -> %d) not supported", h, w);
  tcx_params prm;
  memset(&prm, 0, sizeof(prm));
  for (int c = 0; c < h; c++) {
    prm.x.col[c] = X->col[c];
    if ((uintptr_t)X->col[c] & 15) return gb_fail(ctx, "tc_xc: input column %d not 16-byte aligned", c);
  }
  for (int j = 0; j < w; j++) {
    prm.y.col[j] = Y->col[j];
    if (Z) prm.z.col[j] = Z->col[j];
  }
  prm.C = C;
  prm.ldc = ldc;
  prm.h = h;
  prm.w = w;
  prm.has_z = Z != NULL;
  prm.n = n;
  int* err = (int*)gb_workspace(ctx, 256);
  if (!err) return -1;
  prm.err = err;
  if (cudaMemsetAsync(err, 0, sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "tc_xc: memset failed");
  const long ntiles = (n + 127) / 128;
  const int nctas = (int)(ntiles < ctx->num_sms ? ntiles : ctx->num_sms);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_TC_XC);
  const int rc = w <= 32 ? tcx_launch<32>(ctx, prm, nctas) : tcx_launch<64>(ctx, prm, nctas);
  gb_prof_end(ctx, &pr, 4.0 * n * (h + w + (Z ? w : 0)), 3.0 * 2.0 * n * h * w);
  gb_count_launch(1);
  if (rc) return rc;
  // a timed-out wait is reported through the context's device error word
  tcx_check_kernel<<<1, 1, 0, (cudaStream_t)ctx->stream>>>(err, ctx->dcount + 5);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "tc_xc_check");
}

extern "C" int gb_device_error(gpu_Context* ctx, int* err)
{
  int* h = (int*)gb_pinned(ctx, sizeof(int));
  if (!h || gb_memcpy_d2h(ctx, h, ctx->dcount + 5, sizeof(int))) return -1;
  *err = *h;
  if (*h && cudaMemsetAsync(ctx->dcount + 5, 0, sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "device error word: memset failed");
  return 0;
}

extern "C" int gpu_ContextDeviceError(gpu_Context* ctx, int* code)
{
  *code = 0;
  return gb_device_error(ctx, code);
}

// ------------------------------------------------------- C-ABI entry point
extern "C" int gpu_BlockUpdate(gpu_MultiVector* X, const double* C_host, int ldc, gpu_MultiVector* Y,
                               gpu_MultiVector* Z, int mode)
{
  gpu_Context* ctx = X->ctx;
  const int h = X->num_active, w = Y->num_active;
  if (ldc < h) return gb_fail(ctx, "BlockUpdate: ldc < h");
  if (Z && Z->num_active != w) return gb_fail(ctx, "BlockUpdate: Z width differs from Y");
  if (mode == 2) {
    if (X->dtype != GPU_MV_FLOAT64 || Y->dtype != GPU_MV_FLOAT64)
      return gb_fail(ctx, "BlockUpdate: mode 2 needs FP64 X and Y");
  } else if (X->dtype != Y->dtype || (Z && Z->dtype != Y->dtype)) {
    return gb_fail(ctx, "BlockUpdate: mixed precisions");
  }
  if (mode == 1 && X->dtype != GPU_MV_FLOAT32) return gb_fail(ctx, "BlockUpdate: mode 1 needs FP32 blocks");
  if (h == 0 || w == 0) return 0;
  blk_cols cx, cy, cz;
  gb_mv_fill_cols(X, &cx, 0);
  gb_mv_fill_cols(Y, &cy, 0);
  if (Z) gb_mv_fill_cols(Z, &cz, 0);
  double* C = (double*)gb_device_alloc(ctx, sizeof(double) * (size_t)ldc * w);
  if (!C) return -1;
  int rc = gb_memcpy_h2d(ctx, C, C_host, sizeof(double) * (size_t)ldc * w);
  if (!rc) {
    if (mode == 0)
      rc = gb_bymat(ctx, X->dtype, X->size, &cx, h, C, ldc, &cy, w, Z ? &cz : NULL);
    else if (mode == 1)
      rc = gb_tc_xc(ctx, X->size, &cx, h, C, ldc, &cy, w, Z ? &cz : NULL);
    else
      rc = gb_oz_xc(ctx, X->size, &cx, h, C, ldc, &cy, w, Z ? &cz : NULL, Z ? Z->dtype : 0, NULL);
  }
  int err = 0;
  if (!rc) rc = gb_device_error(ctx, &err);
  if (!rc && err) rc = gb_fail(ctx, "BlockUpdate: tensor-core kernel timed out (code %d)", err);
  gb_sync(ctx);
  gb_device_free(C);
  return rc;
}
