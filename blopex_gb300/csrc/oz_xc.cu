// oz_xc.cu -- FP64-accurate block update Y = X C (+ Z) on the tensor cores by
// error-free splitting (oz_common.cuh): X an FP64 block of n rows and h <= 64
// columns, C the FP64 h x w coordinate block (w <= 64) on the device, Z an
// optional FP32 or FP64 block, Y FP64 (and optionally its FP32 shadow Y32).
// It is serial_Multi_VectorByMatrix (blopex_serial_double/multivector/
// multi_vector.c:474-524, reached through lobpcg.c:1256-1272: X = X C_X + P,
// AX = AX C_X + AP) with FP64 accuracy for the mixed mode's FP64 blocks.
//
// Scales: each row of X (its h values) and each column of C share one
// power of two; both are cut into S = 6 7-bit digits (42 fraction bits): the
// 42-bit fixed point integer of an X value is split into three exact 14-bit
// halves held as floats, each cut into two digits with FP32 arithmetic.
// Level L = t + u of the digit products is accumulated exactly in FP32 in
// TMEM (|sum| < 2^22 for h <= 64); the epilogue recombines the levels in
// integers (pairs in 32 bits, then 64), converts that exact integer to FP64
// once, scales it by a power of two on the exponent field and adds Z: two
// roundings, at most one unit in the last place (measured faster here than
// an integer-only rounding and alignment of Z, whose dependency chain is
// long).
//
// Per CTA (one per SM, persistent over 128-row tiles; a tile's output columns
// are taken 32 at a time, "units", into two alternating TMEM accumulator sets
// so the MMAs of one unit overlap the epilogue of the previous one):
//   warp 1      bulk-copies the tile's h columns (128 FP64 rows each, one
//               cp.async.bulk per column) into a raw buffer, and prefetches
//               the next tile's columns into L2;
//   warps 2-3, 12-15  find each row's scale and write the S digit slices
//               of the tile in the 128-byte-swizzled K-major layout (row =
//               block row, K = the h columns);
//   warp 0      allocates TMEM; one thread issues tcgen05.mma.kind::f16
//               (M = 128, K = 16): for X slice t one MMA per K step against
//               the C slices 0 .. S-1-t stacked along N (N = 32 (S - t)), so
//               level t + v lands at TMEM column 32 (t + v);
//   warps 4-11  read a unit's S level accumulators (lane = row; warps w and
//               w + 4 share TMEM lanes and take 16 of the unit's 32 columns
//               each), recombine and store Y (and Y32).
// Every wait is bounded; a timeout sets an error word and all roles finish.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "internal.h"
#include "oz_common.cuh"

#define OZX_S 6
#define OZX_F (7 * OZX_S)
#define OZX_THREADS 512
#define OZX_NPROD 192
#define OZX_ASLICE 16384          // 128 rows x 128 bytes
#define OZX_BSLICE 4096           // 32 rows x 128 bytes (one unit's columns of one slice)
#define OZX_UNIT 32               // output columns per unit
#define OZX_SET (OZX_S * OZX_UNIT)  // TMEM columns of one accumulator set
#define OZX_C_BYTES (2 * OZX_S * OZX_BSLICE)  // [unit half][slice][32 rows][128 B]
#define OZX_A_BYTES (OZX_S * OZX_ASLICE)
#define OZX_RAW_BYTES (64 * 1024)   // 64 columns x 128 FP64 rows
#define OZX_SMEM (OZX_C_BYTES + OZX_A_BYTES + OZX_RAW_BYTES + 1024)

struct ozx_params {
  blk_cols x, y, z, y32;
  const double* C;
  int ldc, h, w, z_kind;  // z_kind: 0 none, 1 FP32, 2 FP64
  int has_y32;
  long n;
  int* err;
};

// the six digits of an X value (42-bit fixed point against its row's scale
// E) with FP32 arithmetic: three exact 14-bit halves, two digits each
static __device__ __forceinline__ void ozx_digits(double v, int E, float (&d)[OZX_S])
{
  const uint64_t U = oz_fixed64<OZX_F>(v, E);  // <= 2^42
  const uint32_t sg = (uint32_t)((uint64_t)__double_as_longlong(v) >> 63) << 31;
  const uint32_t part[3] = {(uint32_t)(U >> 28), (uint32_t)(U >> 14) & 0x3FFFu, (uint32_t)U & 0x3FFFu};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const float c = __uint_as_float(__float_as_uint(__uint_as_float(0x4B000000u | part[q]) - 8388608.0f) ^ sg);
    d[2 * q] = fmaf(c, 0.0078125f, OZ_RINT_MAGIC) - OZ_RINT_MAGIC;  // in [-128, 128]
    d[2 * q + 1] = fmaf(d[2 * q], -128.0f, c);                        // in [-64, 64]
  }
}

// the Z values of one row in columns j0 .. j0 + 7 (bit patterns; 0 outside)
static __device__ __forceinline__ void ozx_load_z(int z_kind, const void* const* s_z, int j0, int w, long row,
                                                  long n, unsigned long long (&zb)[8])
{
#pragma unroll
  for (int jj = 0; jj < 8; jj++) {
    const int j = j0 + jj;
    zb[jj] = 0;
    if (j0 >= 0 && row < n && j < w) {
      if (z_kind == 1)
        zb[jj] = __float_as_uint(((const float*)s_z[j])[row]);
      else if (z_kind == 2)
        zb[jj] = (unsigned long long)__double_as_longlong(((const double*)s_z[j])[row]);
    }
  }
}

__global__ void __launch_bounds__(OZX_THREADS, 1) oz_xc_kernel(const __grid_constant__ ozx_params prm)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_align1024(smem_raw);
  unsigned char* cdig = smem;                    // [half][S][32 rows][128 B]
  unsigned char* adig = smem + OZX_C_BYTES;      // [S][128 rows][128 B]
  double* raw = (double*)(adig + OZX_A_BYTES);   // [64 columns][128 rows]
  __shared__ uint64_t raw_full, raw_empty, a_full, a_empty, acc_full[2], acc_empty[2], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ int colexp[64];
  __shared__ int rowexp[4][128];   // by tile modulo 4 (read by the epilogue)
  __shared__ int rowpart[8][128];  // per (8-column group, row) largest exponent
  // column pointers: shared memory serves a runtime index in a few cycles,
  // where the kernel-parameter table behind it (four 3 KB arrays) does not
  __shared__ const void* s_x[64];
  __shared__ void* s_y[64];
  __shared__ const void* s_z[64];
  __shared__ void* s_y32[64];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int h = prm.h, w = prm.w;
  const int ksteps = (h + 15) >> 4;
  const int nh = (w + OZX_UNIT - 1) / OZX_UNIT;  // units per tile
  const long ntiles = (prm.n + 127) / 128;
  const long my_tiles = (long)blockIdx.x < ntiles ? (ntiles - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  if (tid == 0) {
    abort_flag = 0;
    mbar_init(&raw_full, 1);
    mbar_init(&raw_empty, OZX_NPROD);
    mbar_init(&a_full, OZX_NPROD);
    mbar_init(&a_empty, 1);
    for (int b = 0; b < 2; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 256);
    }
    mbar_init(&done_bar, 1);
  }
  if (tid < 64) {
    s_x[tid] = tid < h ? prm.x.col[tid] : nullptr;
    s_y[tid] = tid < w ? (void*)prm.y.col[tid] : nullptr;
    s_z[tid] = (tid < w && prm.z_kind) ? prm.z.col[tid] : nullptr;
    s_y32[tid] = (tid < w && prm.has_y32) ? (void*)prm.y32.col[tid] : nullptr;
  }
  // C: one scale per column, digits as the B operand (row j = output column,
  // K = input column); rows j >= w and columns i >= h are zero
  for (int j = tid; j < 64; j += OZX_THREADS) {
    int e = 0;
    if (j < w)
#pragma unroll 8
      for (int i = 0; i < h; i++) e = max(e, oz_bexp64(prm.C[i + (size_t)j * prm.ldc]));
    colexp[j] = e;
  }
  __syncthreads();
  for (int e = tid; e < 64 * 8; e += OZX_THREADS) {  // (row j, 8-column group cg)
    const int j = e % 64, cg = e / 64;
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
    // rows of one unit half hold its 32 output columns; within a half the
    // slices are stacked, so one MMA can take the slices v = 0 .. S-1-t as a
    // single N = 32 (S - t) operand
    const int jr = j & 31, hf = j >> 5;
    const uint32_t off = (uint32_t)jr * 128u + ((uint32_t)(cg ^ (jr & 7)) << 4);
#pragma unroll
    for (int t = 0; t < OZX_S; t++)
      *(uint4*)(cdig + (hf * OZX_S + t) * OZX_BSLICE + off) = make_uint4(p[t][0], p[t][1], p[t][2], p[t][3]);
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"(512u)
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
        bulk_g2s(raw + c * 128, (const double*)s_x[c] + r0, bytes, &raw_full);
      issued = i + 1;
      // the next tile's columns on their way into L2 while this one is cut
      if (i + 1 < my_tiles) {
        const long r1 = r0 + (long)gridDim.x * 128;
        const long rows1 = min(128L, prm.n - r1);
        const uint32_t b1 = (uint32_t)(((rows1 + 1) & ~1L) * 8);
        for (int c = lane; c < h; c += 32)
          asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((const double*)s_x[c] + r1),
                       "r"(b1)
                       : "memory");
      }
    }
    // no copy may still be landing when the CTA exits
    if (issued > 0) mbar_drain(&raw_full, (uint32_t)((issued - 1) & 1));
  } else if (warp == 2 || warp == 3 || warp >= 12) {
    // ------------------------------------------------------- digit slices
    // (every producer runs every iteration: the named barriers below must
    // be reached by all of them; an abort only skips the work).  Work unit
    // (row r, 8-column group cg); 32 consecutive rows per warp.
    const int p = (warp < 4 ? warp - 2 : warp - 10) * 32 + lane;
    for (long i = 0; i < my_tiles; i++) {
      if (!abort_flag && !mbar_wait(&raw_full, (uint32_t)(i & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 12);
      }
      const long r0 = (blockIdx.x + i * gridDim.x) * 128;
      // pass 1: largest exponent of each (group, row)
      for (int uu = p; uu < 1024; uu += OZX_NPROD) {
        const int r = uu & 127, cg = uu >> 7;
        int e = 0;
        if (r0 + r < prm.n && !abort_flag)
#pragma unroll
          for (int c = 0; c < 8; c++)
            if (cg * 8 + c < h) e = max(e, oz_bexp64(raw[(cg * 8 + c) * 128 + r]));
        rowpart[cg][r] = e;
      }
      named_bar(1, OZX_NPROD);
      // the A slices are free once the previous tile's MMAs have completed
      if (i >= 1 && !abort_flag && !mbar_wait(&a_empty, (uint32_t)((i - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 13);
      }
      if (!abort_flag) {
        tc_fence_after();
        // pass 2: the digits of (row r, columns 8 cg .. 8 cg + 7)
        for (int uu = p; uu < 1024; uu += OZX_NPROD) {
          const int r = uu & 127, cg = uu >> 7;
          const bool valid = r0 + r < prm.n;
          int e = 0;
#pragma unroll
          for (int g = 0; g < 8; g++) e = max(e, rowpart[g][r]);
          float dg[8][OZX_S];
#pragma unroll
          for (int c = 0; c < 8; c++) {
            const int col = cg * 8 + c;
            ozx_digits((valid && col < h) ? raw[col * 128 + r] : 0.0, e, dg[c]);
          }
          const uint32_t off = (uint32_t)r * 128u + ((uint32_t)(cg ^ (r & 7)) << 4);
#pragma unroll
          for (int t = 0; t < OZX_S; t++)
            *(uint4*)(adig + t * OZX_ASLICE + off) =
                make_uint4(oz_pack_bf16(dg[0][t], dg[1][t]), oz_pack_bf16(dg[2][t], dg[3][t]),
                           oz_pack_bf16(dg[4][t], dg[5][t]), oz_pack_bf16(dg[6][t], dg[7][t]));
          if (cg == 0) rowexp[i & 3][r] = valid ? e : 0;
        }
        fence_proxy_async();
        mbar_arrive(&a_full);
        mbar_arrive(&raw_empty);
      }
      named_bar(1, OZX_NPROD);  // rowpart is rewritten by the next tile's pass 1
    }
  } else if (warp == 0 && lane == 0) {
    // ------------------------------------------------------- MMA issuer
    const uint32_t abase = smem_u32(adig), cbase = smem_u32(cdig);
    long u = 0;  // units issued
    for (long i = 0; i < my_tiles && !abort_flag; i++) {
      if (!mbar_wait(&a_full, (uint32_t)(i & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 14);
        break;
      }
      for (int hf = 0; hf < nh; hf++, u++) {
        const int set = (int)(u & 1);
        if (u >= 2 && !mbar_wait(&acc_empty[set], (uint32_t)(((u >> 1) - 1) & 1), &abort_flag)) {
          abort_flag = 1;
          atomicExch(prm.err, 15);
          break;
        }
        tc_fence_after();
        for (int t = 0; t < OZX_S; t++) {
          const uint32_t d = tmem + (uint32_t)(set * OZX_SET + t * OZX_UNIT);
          const uint32_t idesc = bf16_idesc(128, OZX_UNIT * (OZX_S - t));
          for (int ks = 0; ks < ksteps; ks++)
            mma_bf16(d, sw128_desc(abase + t * OZX_ASLICE + ks * 32),
                     sw128_desc(cbase + hf * OZX_S * OZX_BSLICE + ks * 32), idesc,
                     (t > 0 || ks > 0) ? 1u : 0u);
        }
        mma_commit(&acc_full[set]);
      }
      if (abort_flag) break;
      mma_commit(&a_empty);
    }
    mma_commit(&done_bar);
  } else if (warp >= 4 && warp < 12) {
    // ------------------------------------------------------- epilogue
    const int quarter = warp & 3, chalf = (warp - 4) >> 2;
    const int r = 32 * quarter + lane;
    long u = 0;
    bool stop = false;
    unsigned long long zn[8];  // the next column group's Z values
    for (long i = 0; i < my_tiles && !stop; i++) {
      const long row = (blockIdx.x + i * gridDim.x) * 128 + r;
      for (int hf = 0; hf < nh; hf++, u++) {
        const int set = (int)(u & 1);
        const int jbase = hf * OZX_UNIT + 16 * chalf;  // this warp's 16 columns
        ozx_load_z(prm.z_kind, s_z, jbase, w, row, prm.n, zn);
        const bool got = mbar_wait(&acc_full[set], (uint32_t)((u >> 1) & 1), &abort_flag);
        if (!__all_sync(0xffffffffu, got)) {  // tcgen05.ld needs the whole warp
          abort_flag = 1;
          atomicExch(prm.err, 16);
          stop = true;
          break;
        }
        tc_fence_after();
        const int er = rowexp[i & 3][r];
        const uint32_t tl = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(set * OZX_SET + 16 * chalf);
#pragma unroll 1
        for (int g = 0; g < 2; g++) {
          const int j0 = jbase + 8 * g;
          unsigned long long zb[8];
#pragma unroll
          for (int jj = 0; jj < 8; jj++) zb[jj] = zn[jj];
          if (g == 0) ozx_load_z(prm.z_kind, s_z, j0 + 8, w, row, prm.n, zn);
          // the six levels of these 8 columns, one wait
          uint32_t v[OZX_S][8];
#pragma unroll
          for (int L = 0; L < OZX_S; L++)
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                : "=r"(v[L][0]), "=r"(v[L][1]), "=r"(v[L][2]), "=r"(v[L][3]), "=r"(v[L][4]),
                  "=r"(v[L][5]), "=r"(v[L][6]), "=r"(v[L][7])
                : "r"(tl + (uint32_t)(L * OZX_UNIT + 8 * g)));
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
          if (row < prm.n) {
#pragma unroll
            for (int jj = 0; jj < 8; jj++) {
              const int j = j0 + jj;
              if (j >= w) continue;
              // T = sum_L S_L 128^(5-L): level pairs in 32 bits (|S| < 2^22),
              // exact in 64; one conversion to FP64, the scale 2^base on the
              // exponent field, then + Z
              const int a0 = oz_int_of(__uint_as_float(v[0][jj])) * 128 + oz_int_of(__uint_as_float(v[1][jj]));
              const int a1 = oz_int_of(__uint_as_float(v[2][jj])) * 128 + oz_int_of(__uint_as_float(v[3][jj]));
              const int a2 = oz_int_of(__uint_as_float(v[4][jj])) * 128 + oz_int_of(__uint_as_float(v[5][jj]));
              const long long t = ((long long)a0 << 28) + ((long long)a1 << 14) + (long long)a2;
              const int ec = colexp[j];
              double y = 0.0;
              if (t != 0 && er != 0 && ec != 0) {
                const double td = (double)t;  // |t| < 2^57: one rounding
                const long long tb = __double_as_longlong(td);
                const int e = (int)((tb >> 52) & 0x7FF) + er + ec - 2058 - 7 * (OZX_S - 1);
                if (e > 0 && e < 2047) y = __longlong_as_double((tb & ~(0x7FFLL << 52)) | ((long long)e << 52));
              }
              if (prm.z_kind == 1)
                y += (double)__uint_as_float((uint32_t)zb[jj]);
              else if (prm.z_kind == 2)
                y += __longlong_as_double((long long)zb[jj]);
              ((double*)s_y[j])[row] = y;
              if (prm.has_y32) ((float*)s_y32[j])[row] = oz_to_float(y);
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[set]);
      }
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
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512u) : "memory");
  }
}

static int ozx_launch(gpu_Context* ctx, const ozx_params& prm, int nctas)
{
  if (cudaFuncSetAttribute(oz_xc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZX_SMEM) !=
      cudaSuccess)
    return gb_fail(ctx, "oz_xc: cannot reserve %d bytes of shared memory", OZX_SMEM);
  if (tc_apply_wait_polls(ctx->opt.wait_polls, (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "oz_xc: cannot set the wait limit");
  oz_xc_kernel<<<nctas, OZX_THREADS, OZX_SMEM, (cudaStream_t)ctx->stream>>>(prm);
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
  const int rc = ozx_launch(ctx, prm, nctas);
  const double zb = Z ? (z_dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0) * w : 0.0;
  gb_prof_end(ctx, &pr, (double)n * (8.0 * h + 8.0 * w + zb + (Y32 ? 4.0 * w : 0.0)),
              2.0 * n * h * w);
  gb_count_launch(1);
  if (rc) return rc;
  ozx_check_kernel<<<1, 1, 0, (cudaStream_t)ctx->stream>>>(err, ctx->dcount + 5);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "oz_xc_check");
}
