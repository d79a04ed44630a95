// oz_xc.cu -- FP64-accurate block update Y = X C (+ Z) on the tensor cores by
// error-free splitting (oz_common.cuh): X an FP64 block of n rows and h <= 64
// columns, C the FP64 h x w coordinate block (w <= 64) on the device, Z an
// optional FP32 or FP64 block, Y FP64 (and optionally its FP32 shadow Y32).
// It is serial_Multi_VectorByMatrix (blopex_serial_double/multivector/
// multi_vector.c:474-524, reached through lobpcg.c:1256-1272: X = X C_X + P,
// AX = AX C_X + AP) with FP64 accuracy for the mixed mode's FP64 blocks.
//
// Scales: each row of X (its h values) and each column of C share one
// power of two; X rows are cut into S = 6 balanced 7-bit digits (42 fraction
// bits), C columns likewise.  Level L = t + u of the digit products is
// accumulated exactly in FP32 in TMEM (|sum| < 2^21 for h <= 64); the epilogue
// recombines the levels in 64-bit integers, adds Z in the same fixed point
// and rounds once to FP64.
//
// Per CTA (one per SM, persistent over 128-row tiles):
//   warp 1      bulk-copies the tile's h columns (128 FP64 rows each, one
//               cp.async.bulk per column) into a raw buffer;
//   warps 8-15  find each row's scale and write the S digit slices of the
//               tile in the 128-byte-swizzled K-major layout (row = block
//               row, K = the h columns);
//   warp 0      allocates TMEM; one thread issues tcgen05.mma.kind::f16
//               (M = 128, N = NW, K = 16) for the pairs t + u < S;
//   warps 4-7   read the S level accumulators (lane = row), recombine and
//               store Y (and Y32).
// Every wait is bounded; a timeout sets an error word and all roles finish.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "internal.h"
#include "oz_common.cuh"

#define OZX_S 6
#define OZX_F (7 * OZX_S)
#define OZX_THREADS 512
#define OZX_NPROD 256
#define OZX_ASLICE 16384  // 128 rows x 128 bytes
static_assert(OZX_S % 3 == 0, "the epilogue reads the levels three at a time");

struct ozx_params {
  blk_cols x, y, z, y32;
  const double* C;
  int ldc, h, w, z_kind;  // z_kind: 0 none, 1 FP32, 2 FP64
  int has_y32;
  long n;
  int* err;
};

template <int NW>
struct ozx_cfg {
  static constexpr int BSLICE = NW * 128;
  static constexpr int C_BYTES = OZX_S * BSLICE;
  static constexpr int A_BYTES = OZX_S * OZX_ASLICE;
  static constexpr int RAW_BYTES = 64 * 1024;  // 64 columns x 128 FP64 rows
  static constexpr int SMEM = C_BYTES + A_BYTES + RAW_BYTES + 1024;
  static constexpr int TMEM_COLS = OZX_S * NW <= 256 ? 256 : 512;
};

// store 8 digits-per-slice of one (row, 8-column group) into the A slices
static __device__ __forceinline__ void ozx_put(unsigned char* adig, int r, int cg, const uint32_t (&p)[OZX_S][4])
{
  const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(cg ^ (r & 7)) << 4);
#pragma unroll
  for (int t = 0; t < OZX_S; t++) *(uint4*)(adig + t * OZX_ASLICE + off) = make_uint4(p[t][0], p[t][1], p[t][2], p[t][3]);
}

template <int NW>
__global__ void __launch_bounds__(OZX_THREADS, 1) oz_xc_kernel(const __grid_constant__ ozx_params prm)
{
  using G = ozx_cfg<NW>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* cdig = smem;                 // [S][NW rows][128 B]
  unsigned char* adig = smem + G::C_BYTES;    // [S][128 rows][128 B]
  double* raw = (double*)(adig + G::A_BYTES);  // [64 columns][128 rows]
  __shared__ uint64_t raw_full, raw_empty, a_full, a_empty, acc_full, acc_empty, done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag, never_flag;
  __shared__ int colexp[64];
  __shared__ int rowexp[2][128];
  __shared__ int rowpart[2][128];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int h = prm.h, w = prm.w;
  const int ksteps = (h + 15) >> 4;
  const long ntiles = (prm.n + 127) / 128;
  const long my_tiles = (long)blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  if (tid == 0) {
    abort_flag = 0;
    never_flag = 0;
    mbar_init(&raw_full, 1);
    mbar_init(&raw_empty, OZX_NPROD);
    mbar_init(&a_full, OZX_NPROD);
    mbar_init(&a_empty, 1);
    mbar_init(&acc_full, 1);
    mbar_init(&acc_empty, 128);
    mbar_init(&done_bar, 1);
  }
  // C: one scale per column, digits as the B operand (row j = output column,
  // K = input column); rows j >= w and columns i >= h are zero
  for (int j = tid; j < 64; j += OZX_THREADS) {
    int e = 0;
    if (j < w)
      for (int i = 0; i < h; i++) e = max(e, oz_bexp64(prm.C[i + (size_t)j * prm.ldc]));
    colexp[j] = e;
  }
  __syncthreads();
  for (int e = tid; e < NW * 8; e += OZX_THREADS) {  // (row j, 8-column group cg)
    const int j = e % NW, cg = e / NW;
    uint32_t p[OZX_S][4];
#pragma unroll
    for (int c = 0; c < 8; c += 2) {
      uint32_t d0[OZX_S], d1[OZX_S];
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int i = cg * 8 + c + q;
        const double v = (j < w && i < h) ? prm.C[i + (size_t)j * prm.ldc] : 0.0;
        const uint64_t U = oz_fixed64<OZX_F>(v, colexp[j]);
        const uint32_t neg = (uint32_t)((uint64_t)__double_as_longlong(v) >> 63);
        if (q == 0)
          oz_digits<OZX_S>(U, neg, d0);
        else
          oz_digits<OZX_S>(U, neg, d1);
      }
#pragma unroll
      for (int t = 0; t < OZX_S; t++) p[t][c >> 1] = d0[t] | (d1[t] << 16);
    }
    const uint32_t off = (uint32_t)j * 128u + ((uint32_t)(cg ^ (j & 7)) << 4);
#pragma unroll
    for (int t = 0; t < OZX_S; t++)
      *(uint4*)(cdig + t * G::BSLICE + off) = make_uint4(p[t][0], p[t][1], p[t][2], p[t][3]);
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

  if (warp == 1) {
    // ------------------------------------------------------- bulk copies
    long issued = 0;
    for (long i = 0; i < my_tiles; i++) {
      int stop = 0;
      if (lane == 0) {
        if (i >= 1 && !mbar_wait(&raw_empty, (uint32_t)((i - 1) & 1), &abort_flag)) {
          abort_flag = 1;
          atomicExch(prm.err, 11);
        }
        stop = abort_flag;
      }
      if (__shfl_sync(0xffffffffu, stop, 0)) break;
      const long r0 = (blockIdx.x + i * gridDim.x) * 128;
      const long rows = min(128L, prm.n - r0);
      const uint32_t bytes = (uint32_t)(((rows + 1) & ~1L) * 8);  // whole 16-byte pieces
      if (lane == 0) mbar_expect_tx(&raw_full, bytes * (uint32_t)h);
      __syncwarp();
      for (int c = lane; c < h; c += 32)
        bulk_g2s(raw + c * 128, (const double*)prm.x.col[c] + r0, bytes, &raw_full);
      issued = i + 1;
    }
    // no copy may still be landing when the CTA exits
    if (issued > 0) mbar_wait(&raw_full, (uint32_t)((issued - 1) & 1), &never_flag);
  } else if (warp >= 8) {
    // ------------------------------------------------------- digit slices
    // (every producer runs every iteration: the named barriers below must
    // be reached by all of them; an abort only skips the work)
    const int p = tid - 256;
    const int r = p & 127, half = p >> 7;
    for (long i = 0; i < my_tiles; i++) {
      if (!abort_flag && !mbar_wait(&raw_full, (uint32_t)(i & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 12);
      }
      const long r0 = (blockIdx.x + i * gridDim.x) * 128;
      const bool valid = r0 + r < prm.n;
      int* part = rowpart[i & 1];
      // the row's scale: largest exponent over its h values
      int e = 0;
      if (valid && !abort_flag)
        for (int c = half * 32; c < min(h, half * 32 + 32); c++) e = max(e, oz_bexp64(raw[c * 128 + r]));
      if (half) part[r] = e;
      named_bar(1, OZX_NPROD);
      if (!half) part[r] = max(e, part[r]);
      named_bar(1, OZX_NPROD);
      e = part[r];
      // the A slices are free once the previous tile's MMAs have completed
      if (i >= 1 && !abort_flag && !mbar_wait(&a_empty, (uint32_t)((i - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 13);
      }
      if (abort_flag) continue;
      tc_fence_after();
      for (int cg = half; cg < 8; cg += 2) {
        uint32_t pk[OZX_S][4];
#pragma unroll
        for (int c = 0; c < 8; c += 2) {
          uint32_t d0[OZX_S], d1[OZX_S];
#pragma unroll
          for (int q = 0; q < 2; q++) {
            const int col = cg * 8 + c + q;
            const double v = (valid && col < h) ? raw[col * 128 + r] : 0.0;
            const uint64_t U = oz_fixed64<OZX_F>(v, e);
            const uint32_t neg = (uint32_t)((uint64_t)__double_as_longlong(v) >> 63);
            if (q == 0)
              oz_digits<OZX_S>(U, neg, d0);
            else
              oz_digits<OZX_S>(U, neg, d1);
          }
#pragma unroll
          for (int t = 0; t < OZX_S; t++) pk[t][c >> 1] = d0[t] | (d1[t] << 16);
        }
        ozx_put(adig, r, cg, pk);
      }
      if (!half) rowexp[i & 1][r] = valid ? e : 0;
      fence_proxy_async();
      mbar_arrive(&a_full);
      mbar_arrive(&raw_empty);
    }
  } else if (warp == 0 && lane == 0) {
    // ------------------------------------------------------- MMA issuer
    const uint32_t idesc = bf16_idesc(128, NW);
    const uint32_t abase = smem_u32(adig), cbase = smem_u32(cdig);
    for (long i = 0; i < my_tiles && !abort_flag; i++) {
      if (!mbar_wait(&a_full, (uint32_t)(i & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 14);
        break;
      }
      if (i >= 1 && !mbar_wait(&acc_empty, (uint32_t)((i - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 15);
        break;
      }
      tc_fence_after();
      for (int t = 0; t < OZX_S; t++)
        for (int u = 0; u + t < OZX_S; u++) {
          const uint32_t d = tmem + (uint32_t)((t + u) * NW);
          for (int ks = 0; ks < ksteps; ks++)
            mma_bf16(d, sw128_desc(abase + t * OZX_ASLICE + ks * 32),
                     sw128_desc(cbase + u * G::BSLICE + ks * 32), idesc, (t > 0 || ks > 0) ? 1u : 0u);
        }
      mma_commit(&a_empty);
      mma_commit(&acc_full);
    }
    mma_commit(&done_bar);
  } else if (warp >= 4 && warp < 8) {
    // ------------------------------------------------------- epilogue
    const int quarter = warp - 4;
    const int r = 32 * quarter + lane;
    for (long i = 0; i < my_tiles; i++) {
      const bool got = mbar_wait(&acc_full, (uint32_t)(i & 1), &abort_flag);
      if (!__all_sync(0xffffffffu, got)) {  // tcgen05.ld needs the whole warp
        abort_flag = 1;
        atomicExch(prm.err, 16);
        break;
      }
      tc_fence_after();
      const long row = (blockIdx.x + i * gridDim.x) * 128 + r;
      const int er = rowexp[i & 1][r];
      const uint32_t tl = tmem + ((uint32_t)(32 * quarter) << 16);
#pragma unroll 1
      for (int g = 0; g < NW / 16; g++) {
        // this row's 16 Z values: all loads in flight before the TMEM reads
        unsigned long long zb[16];
#pragma unroll
        for (int jj = 0; jj < 16; jj++) {
          const int j = 16 * g + jj;
          zb[jj] = 0;
          if (row < prm.n && j < w) {
            if (prm.z_kind == 1)
              zb[jj] = __float_as_uint(((const float*)prm.z.col[j])[row]);
            else if (prm.z_kind == 2)
              zb[jj] = (unsigned long long)__double_as_longlong(((const double*)prm.z.col[j])[row]);
          }
        }
        long long T[16];
#pragma unroll
        for (int jj = 0; jj < 16; jj++) T[jj] = 0;
        // the S level accumulators of these 16 columns, two waits in all
#pragma unroll
        for (int L0 = 0; L0 < OZX_S; L0 += 3) {
          uint32_t v[3][16];
#pragma unroll
          for (int L = 0; L < 3; L++)
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,"
                "%13,%14,%15}, [%16];"
                : "=r"(v[L][0]), "=r"(v[L][1]), "=r"(v[L][2]), "=r"(v[L][3]), "=r"(v[L][4]),
                  "=r"(v[L][5]), "=r"(v[L][6]), "=r"(v[L][7]), "=r"(v[L][8]), "=r"(v[L][9]),
                  "=r"(v[L][10]), "=r"(v[L][11]), "=r"(v[L][12]), "=r"(v[L][13]), "=r"(v[L][14]),
                  "=r"(v[L][15])
                : "r"(tl + (uint32_t)((L0 + L) * NW + 16 * g)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int L = 0; L < 3; L++)
#pragma unroll
            for (int jj = 0; jj < 16; jj++) T[jj] = T[jj] * 128 + oz_int_of(__uint_as_float(v[L][jj]));
        }
        if (row < prm.n) {
#pragma unroll
          for (int jj = 0; jj < 16; jj++) {
            const int j = 16 * g + jj;
            if (j >= w) continue;
            long long mz = 0;
            int ez = 0;
            if (prm.z_kind == 1)
              oz_unpack32(__uint_as_float((uint32_t)zb[jj]), mz, ez);
            else if (prm.z_kind == 2)
              oz_unpack64(__longlong_as_double((long long)zb[jj]), mz, ez);
            const int ec = colexp[j];
            double y;
            if (er == 0 || ec == 0) {
              y = mz ? oz_to_double(mz, ez) : 0.0;
            } else {
              long long t = T[jj];
              int base = er + ec - 2058 - 7 * (OZX_S - 1);
              if (mz) {
                const int dmax = prm.z_kind == 2 ? 8 : 37;  // keeps |z| below 2^61 in T's units
                int d = ez - base;
                if (d > dmax) {
                  const int s = d - dmax;
                  t = s >= 63 ? 0 : ((t + (1LL << (s - 1))) >> s);
                  base += s;
                  d = dmax;
                }
                long long za;
                if (d >= 0)
                  za = mz << d;
                else
                  za = -d >= 63 ? 0 : ((mz + (1LL << (-d - 1))) >> -d);
                t += za;
              }
              y = oz_to_double(t, base);
            }
            ((double*)prm.y.col[j])[row] = y;
            if (prm.has_y32) ((float*)prm.y32.col[j])[row] = oz_to_float(y);
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty);
    }
  }
  // TMEM is freed only after the last MMA has completed (done_bar is always
  // committed by the issuer) and every epilogue read has finished
  if (warp == 0) {
    mbar_wait(&done_bar, 0, &never_flag);
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
static int ozx_launch(gpu_Context* ctx, const ozx_params& prm, int nctas)
{
  const int smem = ozx_cfg<NW>::SMEM;
  if (cudaFuncSetAttribute(oz_xc_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return gb_fail(ctx, "oz_xc: cannot reserve %d bytes of shared memory", smem);
  oz_xc_kernel<NW><<<nctas, OZX_THREADS, smem, (cudaStream_t)ctx->stream>>>(prm);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "oz_xc");
}

__global__ void ozx_check_kernel(const int* err, int* status)
{
  if (*err) *status = *err;
}

extern "C" int gb_oz_xc(gpu_Context* ctx, long n, const blk_cols* X, int h, const double* C, int ldc,
                        const blk_cols* Y, int w, const blk_cols* Z, int z_dtype, const blk_cols* Y32)
{
  if (n <= 0 || w <= 0) return 0;
  if (h < 1 || h > 64 || w > 64)
    return gb_fail(ctx, "oz_xc: block widths (%d -> %d) not supported", h, w);
  ozx_params prm;
  memset(&prm, 0, sizeof(prm));
  for (int c = 0; c < h; c++) {
    prm.x.col[c] = X->col[c];
    if ((uintptr_t)X->col[c] & 15) return gb_fail(ctx, "oz_xc: input column %d not 16-byte aligned", c);
  }
  for (int j = 0; j < w; j++) {
    prm.y.col[j] = Y->col[j];
    if (Z) prm.z.col[j] = Z->col[j];
    if (Y32) prm.y32.col[j] = Y32->col[j];
  }
  prm.C = C;
  prm.ldc = ldc;
  prm.h = h;
  prm.w = w;
  prm.z_kind = Z ? (z_dtype == GPU_MV_FLOAT64 ? 2 : 1) : 0;
  prm.has_y32 = Y32 != NULL;
  prm.n = n;
  int* err = (int*)gb_workspace(ctx, 256);
  if (!err) return -1;
  prm.err = err;
  if (cudaMemsetAsync(err, 0, sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "oz_xc: memset failed");
  const long ntiles = (n + 127) / 128;
  const int nctas = (int)(ntiles < ctx->num_sms ? ntiles : ctx->num_sms);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_OZ_XC);
  const int rc = w <= 32 ? ozx_launch<32>(ctx, prm, nctas) : ozx_launch<64>(ctx, prm, nctas);
  const double zb = Z ? (z_dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0) * w : 0.0;
  gb_prof_end(ctx, &pr, (double)n * (8.0 * h + 8.0 * w + zb + (Y32 ? 4.0 * w : 0.0)),
              2.0 * n * h * w);
  gb_count_launch(1);
  if (rc) return rc;
  ozx_check_kernel<<<1, 1, 0, (cudaStream_t)ctx->stream>>>(err, ctx->dcount + 5);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "oz_xc_check");
}
