// oz_gram.cu -- FP64-accurate Gram products G = L' [L Q_0 Q_1 ...] on the
// tensor cores by error-free splitting (oz_common.cuh): L a block of h <= 64
// FP32 or FP64 columns, Q_b blocks of up to 64 FP32 or FP64 columns.  It is
// serial_Multi_VectorInnerProd (blopex_serial_double/multivector/
// multi_vector.c:354-406; the Gram blocks of lobpcg.c:1092-1160) with exact
// accumulation: FP32 tensor-core accumulators round toward zero, and summed
// over millions of rows that bias is ~1e-5 relative; the mixed mode's pencil
// breaks down (its R block stops being definite) with biased errors of 1e-6,
// while unbiased errors of 1e-7 leave its convergence that of FP64.
//
// The contraction runs over n rows in chunks of 64.  Within a chunk every
// column has its own power-of-two scale and is cut into S = 4 8-bit digits
// (32 fraction bits; FP32 arithmetic, oz_digits4x8_*); level L = t + u of the
// digit products is summed exactly in FP32 in TMEM (|sum| < 2^24 over 64
// rows: 8 bits per digit is the widest that holds).  After each chunk the four
// levels are combined (FP32, round to nearest), scaled, and added into
// double-float (hi + lo FP32) accumulators, so the chunk sums add without
// bias; each CTA writes its sums in FP64 and a second kernel adds the CTAs
// in a fixed order.
//
// Tile b of the grid pairs L with Q_b: the A operand has 128 rows, L's
// columns in rows 0-63 and Q_b's in rows 64-127; the B operand is rows 0-63
// of the same slices (L).  Per CTA (one per SM):
//   warp 1          copies a chunk's columns into one of two raw buffers:
//                   a run of equally spaced columns (a block's columns at
//                   its leading dimension) as one 2-D TMA tile, other
//                   columns one cp.async.bulk each (the per-request cost of
//                   128 column copies per chunk otherwise bounds the kernel);
//   warps 2-3, 12-15 find each column's chunk scale and write the digit
//                   slices (128-byte-swizzled K-major, K = the chunk's rows);
//   warp 0          allocates TMEM; one thread issues tcgen05.mma.kind::f16
//                   (M = 128, N = 64, K = 16) for the pairs t + u < S into one
//                   of two accumulator sets;
//   warps 4-11      fold a finished chunk into the double-float sums (lane =
//                   column of [L Q_b]; warps w and w + 4 share TMEM lanes and
//                   take 32 of the 64 L columns each).
// Every wait is bounded; a timeout sets an error word, the outputs become NaN.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"
#include "oz_common.cuh"

#define OZG_S 4
#define OZG_F (8 * OZG_S)                // 8-bit digits (oz_digits4x8_*)
#define OZG_THREADS 512
#define OZG_NPROD 192
#define OZG_ROWS 64                      // rows per chunk
// a staged column: 64 rows and 16 bytes more, so that consecutive columns
// start 16 bytes apart modulo 128 (different shared-memory bank groups); a
// TMA tile of 66 FP64 / 68 FP32 rows lands its columns at exactly this stride
#define OZG_STRIDE64 528
#define OZG_STRIDE32 272
#define OZG_RAW 69632                    // one raw buffer: 128 columns + run alignment
#define OZG_SLICE 16384                  // 128 operand rows x 128 bytes
#define OZG_SMEM (2 * OZG_RAW + OZG_S * OZG_SLICE + 1024)
#define OZG_MAXQ 4  // 64 + 64 * OZG_MAXQ column slots fit blk_cols
#define OZG_MAXMAPS 12

struct ozg_params {
  CUtensorMap maps[OZG_MAXMAPS];  // 2-D tiles (rows x columns) of equally spaced column runs
  blk_cols cols;       // tile b: L column c at cols.col[c]; Q_b column j at cols.col[64 + 64 b + j]
  int h, nq, ldt;                   // ldt: dtype of L (GPU_MV_*)
  int qw[OZG_MAXQ], qdt[OZG_MAXQ];  // widths and dtypes (GPU_MV_*) of the Q blocks
  int nmaps;
  int map_tile[OZG_MAXMAPS];   // the tile a map serves; -1: L, every tile
  int map_slot[OZG_MAXMAPS];   // its first column slot
  int map_bytes[OZG_MAXMAPS];  // bytes one load brings (the whole box)
  unsigned short roff[OZG_MAXQ][128];   // raw-buffer offset of each slot, 16-byte units
  unsigned char by_map[OZG_MAXQ][128];  // 1: the slot arrives with a map's tile
  long n;
  double* partial;  // [tile][cta][128][64]
  int* err;
};

// a kernel parameter block of at most 32,764 bytes; raw buffers that keep the
// digit slices behind them 1024-byte aligned (the MMA descriptors' swizzle
// atom); dynamic plus static shared memory within the 227 KB of a CTA
static_assert(sizeof(ozg_params) <= 32764, "oz_gram parameters exceed the kernel parameter space");
static_assert(OZG_RAW % 1024 == 0, "raw buffers must keep the digit slices 1024-byte aligned");
static_assert(OZG_SMEM + 8192 <= 232448, "oz_gram shared memory exceeds a CTA's 227 KB");

// rows x columns tile of a column run: x = first row, the run's columns all
static __device__ __forceinline__ void ozg_tile_load(uint32_t dst, const CUtensorMap* map, int x, uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"((uint64_t)map), "r"(x), "r"(0), "r"(smem_u32(bar))
      : "memory");
}

static __device__ __forceinline__ int ozg_col_kind(const ozg_params& prm, int b, int j, const void** ptr)
{
  // 0: absent, 1: FP32, 2: FP64
  if (j < 64) {
    if (j >= prm.h) return 0;
    *ptr = prm.cols.col[j];
    return prm.ldt == GPU_MV_FLOAT64 ? 2 : 1;
  }
  const int q = j - 64;
  if (b >= prm.nq || q >= prm.qw[b]) return 0;
  *ptr = prm.cols.col[64 + 64 * b + q];
  return prm.qdt[b] == GPU_MV_FLOAT64 ? 2 : 1;
}

// eight consecutive values of a staged column (16-byte aligned) with 16-byte
// shared-memory loads
static __device__ __forceinline__ void ozg_load8(const unsigned char* src, double (&v)[8])
{
#pragma unroll
  for (int x = 0; x < 4; x++) {
    const double2 d = ((const double2*)src)[x];
    v[2 * x] = d.x;
    v[2 * x + 1] = d.y;
  }
}
static __device__ __forceinline__ void ozg_load8(const unsigned char* src, float (&v)[8])
{
  const float4 a = ((const float4*)src)[0], b = ((const float4*)src)[1];
  v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
}

__global__ void __launch_bounds__(OZG_THREADS, 1) oz_gram_kernel(const __grid_constant__ ozg_params prm)
{
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = smem_align1024(smem_raw);
  unsigned char* raws = smem;                  // [2][OZG_RAW]: columns at s_off
  unsigned char* adig = smem + 2 * OZG_RAW;    // [S][128 rows][128 B]
  __shared__ uint64_t raw_full[2], raw_empty[2], a_full, a_empty, acc_full[2], acc_empty[2], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  // this tile's column pointers and kinds (0 absent, 1 FP32, 2 FP64) in shared
  // memory: a runtime index into the kernel-parameter table is slow
  __shared__ const void* s_col[128];
  __shared__ int s_kind[128];
  __shared__ int s_off[128];   // raw-buffer offset of each column
  __shared__ int s_copy[128];  // the column's own bulk copy: 0 none, 1 FP32, 2 FP64
  __shared__ int cexp[4][128];     // chunk scales, by chunk modulo 4

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int b = blockIdx.y;
  const long nchunks = (prm.n + OZG_ROWS - 1) / OZG_ROWS;
  const long my_chunks = (long)blockIdx.x < nchunks ? (nchunks - blockIdx.x + gridDim.x - 1) / gridDim.x : 0;

  if (tid < 128) {
    const void* ptr = nullptr;
    const int kind = ozg_col_kind(prm, b, tid, &ptr);
    s_kind[tid] = kind;
    s_col[tid] = ptr;
    s_off[tid] = 16 * (int)prm.roff[b][tid];
    s_copy[tid] = prm.by_map[b][tid] ? 0 : kind;
  }
  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < 2; s++) {
      mbar_init(&raw_full[s], 1);
      mbar_init(&raw_empty[s], OZG_NPROD);
      mbar_init(&acc_full[s], 1);
      mbar_init(&acc_empty[s], 256);
    }
    mbar_init(&a_full, OZG_NPROD);
    mbar_init(&a_empty, 1);
    mbar_init(&done_bar, 1);
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
    long issued[2] = {0, 0};  // chunks issued per slot
    int ncol8 = 0, ncol4 = 0;  // FP64 and FP32 columns copied one by one
    for (int j = 0; j < 128; j++) {
      ncol8 += s_copy[j] == 2;
      ncol4 += s_copy[j] == 1;
    }
    uint32_t mapbytes = 0;  // the tiles of this CTA's runs
    for (int m = 0; m < prm.nmaps; m++)
      if (prm.map_tile[m] < 0 || prm.map_tile[m] == b) mapbytes += (uint32_t)prm.map_bytes[m];
    for (long c = 0; c < my_chunks; c++) {
      const int slot = (int)(c & 1);
      int stop = 0;
      if (lane == 0) {
        if (c >= 2 && !mbar_wait(&raw_empty[slot], (uint32_t)(((c >> 1) - 1) & 1), &abort_flag)) {
          abort_flag = 1;
          atomicExch(prm.err, 21);
        }
        stop = abort_flag;
      }
      if (__shfl_sync(0xffffffffu, stop, 0)) break;
      const long r0 = (blockIdx.x + c * gridDim.x) * OZG_ROWS;
      const long rows = min((long)OZG_ROWS, prm.n - r0);
      // every column's copy covers whole 16-byte pieces
      const uint32_t b8 = (uint32_t)(((rows + 1) & ~1L) * 8), b4 = (uint32_t)(((rows + 3) & ~3L) * 4);
      // (a tile counts its whole box, rows past n included: they read as 0)
      const uint32_t total = mapbytes + (uint32_t)ncol8 * b8 + (uint32_t)ncol4 * b4;
      if (lane == 0) mbar_expect_tx(&raw_full[slot], total);
      __syncwarp();
      unsigned char* raw = raws + slot * OZG_RAW;
      for (int m = lane; m < prm.nmaps; m += 32)
        if (prm.map_tile[m] < 0 || prm.map_tile[m] == b)
          ozg_tile_load(smem_u32(raw + s_off[prm.map_slot[m]]), &prm.maps[m], (int)r0, &raw_full[slot]);
      for (int j = lane; j < 128; j += 32) {
        const void* ptr = s_col[j];
        const int kind = s_copy[j];
        if (kind == 2)
          bulk_g2s(raw + s_off[j], (const double*)ptr + r0, b8, &raw_full[slot]);
        else if (kind == 1)
          bulk_g2s(raw + s_off[j], (const float*)ptr + r0, b4, &raw_full[slot]);
      }
      issued[slot] = c + 1;
    }
    // no copy may still be landing when the CTA exits
    for (int s = 0; s < 2; s++)
      if (issued[s] > 0) mbar_drain(&raw_full[s], (uint32_t)(((issued[s] - 1) >> 1) & 1));
  } else if (warp == 2 || warp == 3 || warp >= 12) {
    // ------------------------------------------------------- digit slices
    // (every producer runs every iteration: the named barrier below must be
    // reached by all of them; an abort only skips the work)
    const int p = (warp < 4 ? warp - 2 : warp - 10) * 32 + lane;
    for (long c = 0; c < my_chunks; c++) {
      const int slot = (int)(c & 1);
      if (!abort_flag && !mbar_wait(&raw_full[slot], (uint32_t)((c >> 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 22);
      }
      const long r0 = (blockIdx.x + c * gridDim.x) * OZG_ROWS;
      const int rows = (int)min((long)OZG_ROWS, prm.n - r0);
      const unsigned char* raw = raws + slot * OZG_RAW;
      // pass 1: each column's largest exponent over the chunk.  The eight
      // 8-row groups of column j sit in eight consecutive lanes (every lane
      // of a warp runs the same number of iterations), which combine theirs
      // by shuffles.  Only the maximum matters here, so the lanes read their
      // 16-byte pieces in rotated orders: the eight lanes of a column then
      // touch eight different bank groups.
      for (int u = p; u < 1024; u += OZG_NPROD) {
        const int j = u >> 3, q = u & 7;
        const int kind = abort_flag ? 0 : s_kind[j];
        const int nr = min(8, rows - 8 * q);
        int e = 0;
        if (kind == 2) {
          const unsigned char* src = raw + s_off[j] + 64 * q;
#pragma unroll
          for (int x = 0; x < 4; x++) {
            const int xx = (x + (q >> 1)) & 3;  // rows 2 xx, 2 xx + 1
            const double2 d = *(const double2*)(src + 16 * xx);
            if (2 * xx < nr) e = max(e, oz_bexp64(d.x));
            if (2 * xx + 1 < nr) e = max(e, oz_bexp64(d.y));
          }
        } else if (kind == 1) {
          const unsigned char* src = raw + s_off[j] + 32 * q;
#pragma unroll
          for (int x = 0; x < 2; x++) {
            const int hx = x ^ ((q >> 2) & 1);  // rows 4 hx .. 4 hx + 3
            const float4 f = *(const float4*)(src + 16 * hx);
            if (4 * hx < nr) e = max(e, oz_bexp32(f.x));
            if (4 * hx + 1 < nr) e = max(e, oz_bexp32(f.y));
            if (4 * hx + 2 < nr) e = max(e, oz_bexp32(f.z));
            if (4 * hx + 3 < nr) e = max(e, oz_bexp32(f.w));
          }
        }
        e = max(e, __shfl_xor_sync(0xffffffffu, e, 1));
        e = max(e, __shfl_xor_sync(0xffffffffu, e, 2));
        e = max(e, __shfl_xor_sync(0xffffffffu, e, 4));
        // the chunk scale (absent columns: 0).  Slot c mod 4 was last read by
        // the epilogue of chunk c - 4, which finished before the MMAs of
        // chunk c - 2 started (their accumulator buffer), and those completed
        // before the previous chunk's pass 2 (its a_empty wait)
        if (q == 0) cexp[c & 3][j] = e;
      }
      named_bar(1, OZG_NPROD);
      // the digit slices are free once the previous chunk's MMAs completed
      if (c >= 1 && !abort_flag && !mbar_wait(&a_empty, (uint32_t)((c - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 23);
      }
      if (!abort_flag) {
        tc_fence_after();
        // pass 2: the digits of (column j, rows 8q .. 8q + 7).  Eight
        // consecutive lanes take eight consecutive columns at the same q:
        // the raw column stride (528 or 272, 16 mod 128) and the slices' swizzle
        // then put their 16-byte loads and stores in eight different bank
        // groups.
        for (int u = p; u < 1024; u += OZG_NPROD) {
          const int j = (u & 7) | ((u >> 6) << 3), q = (u >> 3) & 7;
          const int E = cexp[c & 3][j];
          const int kind = s_kind[j];
          // the eight rows' digits with FP32 arithmetic (integer fixed point
          // first for FP64 values, or for FP32 groups whose scale leaves the
          // float range)
          float dg[8][OZG_S];
          const float sc = oz_scale4x8(E);
          const int nr = min(8, rows - 8 * q);
          if (kind == 1) {
            float v[8];
            ozg_load8(raw + s_off[j] + 32 * q, v);
#pragma unroll
            for (int x = 0; x < 8; x++) v[x] = x < nr ? v[x] : 0.0f;
            if (sc != 0.0f) {
#pragma unroll
              for (int x = 0; x < 8; x++) oz_digits4x8_f32(v[x], sc, dg[x]);
            } else {
#pragma unroll
              for (int x = 0; x < 8; x++)
                oz_digits4x8_u(oz_fixed32<OZG_F>(v[x], E), __float_as_uint(v[x]) & 0x80000000u, dg[x]);
            }
          } else if (kind == 2) {
            double v[8];
            ozg_load8(raw + s_off[j] + 64 * q, v);
#pragma unroll
            for (int x = 0; x < 8; x++) oz_digits4x8_f64(x < nr ? v[x] : 0.0, E, dg[x]);
          } else {
#pragma unroll
            for (int x = 0; x < 8; x++)
#pragma unroll
              for (int t = 0; t < OZG_S; t++) dg[x][t] = 0.0f;
          }
          uint32_t pk[OZG_S][4];
#pragma unroll
          for (int t = 0; t < OZG_S; t++)
#pragma unroll
            for (int k = 0; k < 4; k++) pk[t][k] = oz_pack_bf16(dg[2 * k][t], dg[2 * k + 1][t]);
          const uint32_t off = (uint32_t)j * 128u + ((uint32_t)(q ^ (j & 7)) << 4);
#pragma unroll
          for (int t = 0; t < OZG_S; t++)
            *(uint4*)(adig + t * OZG_SLICE + off) = make_uint4(pk[t][0], pk[t][1], pk[t][2], pk[t][3]);
        }
        fence_proxy_async();
        mbar_arrive(&a_full);
        mbar_arrive(&raw_empty[slot]);
      }
      // no barrier here: the next chunk's pass 1 writes another scale slot
      // and reads the other raw buffer
    }
  } else if (warp == 0 && lane == 0) {
    // ------------------------------------------------------- MMA issuer
    const uint32_t idesc = bf16_idesc(128, 64);
    const uint32_t abase = smem_u32(adig);
    for (long c = 0; c < my_chunks && !abort_flag; c++) {
      const int buf = (int)(c & 1);
      if (!mbar_wait(&a_full, (uint32_t)(c & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 24);
        break;
      }
      if (c >= 2 && !mbar_wait(&acc_empty[buf], (uint32_t)(((c >> 1) - 1) & 1), &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 25);
        break;
      }
      tc_fence_after();
      for (int t = 0; t < OZG_S; t++)
        for (int u = 0; u + t < OZG_S; u++) {
          const uint32_t d = tmem + (uint32_t)(buf * 256 + (t + u) * 64);
          for (int ks = 0; ks < 4; ks++)
            mma_bf16(d, sw128_desc(abase + t * OZG_SLICE + ks * 32), sw128_desc(abase + u * OZG_SLICE + ks * 32),
                     idesc, (t > 0 || ks > 0) ? 1u : 0u);
        }
      mma_commit(&a_empty);
      mma_commit(&acc_full[buf]);
    }
    mma_commit(&done_bar);
  } else if (warp >= 4 && warp < 12) {
    // ------------------------------------------------------- epilogue
    const int quarter = warp & 3, ihalf = (warp - 4) >> 2;
    const int j = 32 * quarter + lane;
    float hi[32], lo[32];
#pragma unroll
    for (int i = 0; i < 32; i++) hi[i] = lo[i] = 0.f;
    bool ok = true;
    for (long c = 0; c < my_chunks; c++) {
      const int buf = (int)(c & 1);
      const bool got = mbar_wait(&acc_full[buf], (uint32_t)((c >> 1) & 1), &abort_flag);
      if (!__all_sync(0xffffffffu, got)) {  // tcgen05.ld needs the whole warp
        abort_flag = 1;
        atomicExch(prm.err, 26);
        ok = false;
        break;
      }
      tc_fence_after();
      const int* ce = cexp[c & 3];
      const int ej = ce[j];
      // 2^(E - 1022 - 8) per factor: the digit sums carry 2^-8 per factor
      const float fj = (ej >= 904 && ej <= 1157) ? __uint_as_float((uint32_t)(ej - 1030 + 127) << 23) : 0.f;
      const uint32_t tl = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(buf * 256 + 32 * ihalf);
#pragma unroll
      for (int g = 0; g < 4; g++) {
        // the four level accumulators of these 8 columns, one wait for all
        uint32_t r[OZG_S][8];
#pragma unroll
        for (int L = 0; L < OZG_S; L++)
          asm volatile(
              "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
              : "=r"(r[L][0]), "=r"(r[L][1]), "=r"(r[L][2]), "=r"(r[L][3]), "=r"(r[L][4]),
                "=r"(r[L][5]), "=r"(r[L][6]), "=r"(r[L][7])
              : "r"(tl + (uint32_t)(L * 64 + 8 * g)));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        // levels 1.. by Horner, highest first: rest = sum_{L>=1} S_L 2^(8 - 8 L)
        float rest[8];
#pragma unroll
        for (int x = 0; x < 8; x++) {
          rest[x] = __uint_as_float(r[OZG_S - 1][x]);
#pragma unroll
          for (int L = OZG_S - 2; L >= 1; L--) rest[x] = fmaf(rest[x], 0.00390625f, __uint_as_float(r[L][x]));
        }
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const int ii = 8 * g + x;
          const int ei = ce[32 * ihalf + ii];
          const float fi = (ei >= 904 && ei <= 1157) ? __uint_as_float((uint32_t)(ei - 1030 + 127) << 23) : 0.f;
          const float fij = __fmul_rn(fj, fi);
          // level 0 (an integer below 2^22) scaled exactly, added by a
          // two-sum (hi + a = sum + err exactly; intrinsics: no contraction);
          // the levels below it, 2^-8 smaller, into the low word
          const float a = __fmul_rn(__uint_as_float(r[0][x]), fij);
          const float sum = __fadd_rn(hi[ii], a);
          const float bv = __fsub_rn(sum, hi[ii]);
          const float err = __fadd_rn(__fsub_rn(hi[ii], __fsub_rn(sum, bv)), __fsub_rn(a, bv));
          hi[ii] = sum;
          lo[ii] = fmaf(rest[x], __fmul_rn(fij, 0.00390625f), __fadd_rn(lo[ii], err));
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
      // every 8 chunks: (hi, lo) <- two-sum(hi, lo), so the low word stays
      // small and its own FP32 roundings negligible
      if ((c & 7) == 7) {
#pragma unroll
        for (int i = 0; i < 32; i++) {
          const float sum = __fadd_rn(hi[i], lo[i]);
          const float bv = __fsub_rn(sum, hi[i]);
          lo[i] = __fadd_rn(__fsub_rn(hi[i], __fsub_rn(sum, bv)), __fsub_rn(lo[i], bv));
          hi[i] = sum;
        }
      }
    }
    double* out = prm.partial + ((size_t)b * gridDim.x + blockIdx.x) * 128 * 64 + (size_t)j * 64 + 32 * ihalf;
#pragma unroll
    for (int i = 0; i < 32; i++) out[i] = ok ? (double)hi[i] + (double)lo[i] : 0.0;
  }
  // TMEM is freed only after the last MMA has completed and every epilogue
  // read has finished
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

// G(i, col) for i < h: col < h -> tile 0, operand row col; col in Q_b's
// range -> tile b, operand row 64 + (col - start of Q_b); CTAs summed in order
struct ozg_offsets {
  int q[OZG_MAXQ + 1];
};

__global__ void oz_gram_reduce_kernel(const double* __restrict__ partial, int gx, int h, int nq,
                                      ozg_offsets qoff, int wtot, double* G, int ldg, const int* err,
                                      int* status)
{
  // a timed-out wait is also reported through the context's device error word
  if (blockIdx.x == 0 && threadIdx.x == 0 && *err) *status = *err;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= h * wtot) return;
  const int i = e % h, col = e / h;
  int tile = 0, row = col;
  if (col >= h) {
    for (int q = 0; q < nq; q++)
      if (col >= qoff.q[q] && col < qoff.q[q + 1]) {
        tile = q;
        row = 64 + col - qoff.q[q];
      }
  }
  double s = 0.0;
  const double* p = partial + (size_t)tile * gx * 8192 + (size_t)row * 64 + i;
  for (int x = 0; x < gx; x++) s += p[(size_t)x * 8192];
  if (*err) s = __longlong_as_double(0x7ff8000000000000LL);  // NaN: the caller sees a failed Gram
  G[i + (size_t)col * ldg] = s;
}

// columns from slot s0 equally spaced by a stride that a tensor map can
// take (a multiple of 16 bytes, at least a column's bytes): the run's length
// (1 when the next column breaks it)
static int ozg_run_length(const void* const* col, int s0, int maxlen, long colbytes)
{
  if (maxlen < 2) return 1;
  const intptr_t d = (const char*)col[s0 + 1] - (const char*)col[s0];
  if (d <= 0 || d % 16 || d < colbytes || d >= ((intptr_t)1 << 40)) return 1;
  int r = 2;
  while (r < maxlen && (const char*)col[s0 + r] - (const char*)col[s0 + r - 1] == d) r++;
  return r;
}

// a tensor map of the run of r columns from prm->cols.col[s0] (column slot
// `local` of the tile's staging buffer): tiles of 66 FP64 or 68 FP32 rows by
// r columns (rows past n read as 0); 1 when encoded
static int ozg_encode(PFN_cuTensorMapEncodeTiled_v12000 enc, ozg_params* prm, int tile, int s0, int local, int r,
                      int f64)
{
  if (prm->nmaps >= OZG_MAXMAPS) return 0;
  const int rows_box = f64 ? OZG_STRIDE64 / 8 : OZG_STRIDE32 / 4;
  const cuuint64_t dims[2] = {(cuuint64_t)prm->n, (cuuint64_t)r};
  const cuuint64_t strides[1] = {
      (cuuint64_t)((const char*)prm->cols.col[s0 + 1] - (const char*)prm->cols.col[s0])};
  const cuuint32_t box[2] = {(cuuint32_t)rows_box, (cuuint32_t)r}, es[2] = {1, 1};
  if (enc(&prm->maps[prm->nmaps], f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
          (void*)prm->cols.col[s0], dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return 0;
  prm->map_tile[prm->nmaps] = tile;
  prm->map_slot[prm->nmaps] = local;
  prm->map_bytes[prm->nmaps] = rows_box * r * (f64 ? 8 : 4);
  prm->nmaps++;
  return 1;
}

// the staging layout of every tile: L's columns first at their stride, then
// Q_b's; a run of at least two equally spaced columns becomes one tile load
// (its start 128-byte aligned, as TMA wants), other columns are copied one
// by one (all of them without the CUDA driver's encoder, or for short columns)
static int ozg_layout(gpu_Context* ctx, ozg_params* prm, int ntiles)
{
  PFN_cuTensorMapEncodeTiled_v12000 enc = (PFN_cuTensorMapEncodeTiled_v12000)gb_tensormap_encoder();
  if (prm->n < 128 || prm->n >= (1L << 31) - 128) enc = NULL;  // row coordinates are 32-bit
  prm->nmaps = 0;
  const int lf64 = prm->ldt == GPU_MV_FLOAT64, sl = lf64 ? OZG_STRIDE64 : OZG_STRIDE32;
  int lmap = 0;
  if (enc && prm->h >= 2 && ozg_run_length(prm->cols.col, 0, prm->h, prm->n * (lf64 ? 8 : 4)) == prm->h)
    lmap = ozg_encode(enc, prm, -1, 0, 0, prm->h, lf64);
  for (int t = 0; t < ntiles; t++) {
    for (int c = 0; c < prm->h; c++) {
      prm->roff[t][c] = (unsigned short)(c * sl / 16);
      prm->by_map[t][c] = (unsigned char)lmap;
    }
    long off = ((long)prm->h * sl + 127) & ~127L;
    const int w = t < prm->nq ? prm->qw[t] : 0;
    const int qf64 = t < prm->nq && prm->qdt[t] == GPU_MV_FLOAT64, sq = qf64 ? OZG_STRIDE64 : OZG_STRIDE32;
    for (int j = 0; j < w;) {
      const int s0 = 64 + 64 * t + j;
      const int r = enc ? ozg_run_length(prm->cols.col, s0, w - j, prm->n * (qf64 ? 8 : 4)) : 1;
      const long at = (off + 127) & ~127L;
      if (r >= 2 && at + (long)r * sq <= OZG_RAW && ozg_encode(enc, prm, t, s0, 64 + j, r, qf64)) {
        for (int i = 0; i < r; i++) {
          prm->roff[t][64 + j + i] = (unsigned short)((at + (long)i * sq) / 16);
          prm->by_map[t][64 + j + i] = 1;
        }
        off = at + (long)r * sq;
        j += r;
        continue;
      }
      prm->roff[t][64 + j] = (unsigned short)(off / 16);
      prm->by_map[t][64 + j] = 0;
      off += sq;
      j++;
    }
    if (off > OZG_RAW) return gb_fail(ctx, "oz_gram: tile %d needs %ld bytes of staging", t, off);
  }
  return 0;
}

extern "C" int gb_oz_gram(gpu_Context* ctx, long n, const blk_cols* L, int h, int ldt, int nq,
                          const blk_cols* Q, const int* qw, const int* qdt, double* G, int ldg)
{
  if (h < 1 || h > 64 || nq < 0 || nq > OZG_MAXQ || n <= 0)
    return gb_fail(ctx, "oz_gram: shape (h %d, %d blocks) not supported", h, nq);
  ozg_params prm;
  memset(&prm, 0, sizeof(prm));
  prm.h = h;
  prm.nq = nq;
  prm.ldt = ldt;
  prm.n = n;
  for (int c = 0; c < h; c++) {
    prm.cols.col[c] = L->col[c];
    if ((uintptr_t)L->col[c] & 15) return gb_fail(ctx, "oz_gram: column %d of L not 16-byte aligned", c);
  }
  // consecutive Q blocks of one dtype that fit 64 columns together share a
  // tile (a solve's R and P blocks narrow as columns converge): the output
  // columns keep their order, and every entry's digits and level sums are
  // those of its own column pair, so only the work shrinks
  int wtot = h, mq = 0;
  ozg_offsets qoff;
  for (int q = 0; q < nq; q++) {
    if (qw[q] < 0 || qw[q] > 64) return gb_fail(ctx, "oz_gram: block %d has %d columns", q, qw[q]);
    for (int j = 0; j < qw[q]; j++)
      if ((uintptr_t)Q[q].col[j] & 15)
        return gb_fail(ctx, "oz_gram: column %d of block %d not 16-byte aligned", j, q);
    if (qw[q] == 0) continue;
    if (mq == 0 || prm.qdt[mq - 1] != qdt[q] || prm.qw[mq - 1] + qw[q] > 64) {
      prm.qw[mq] = 0;
      prm.qdt[mq] = qdt[q];
      qoff.q[mq] = wtot;
      mq++;
    }
    for (int j = 0; j < qw[q]; j++) prm.cols.col[64 + 64 * (mq - 1) + prm.qw[mq - 1] + j] = Q[q].col[j];
    prm.qw[mq - 1] += qw[q];
    wtot += qw[q];
  }
  nq = mq;
  prm.nq = nq;
  qoff.q[nq] = wtot;
  const int ntiles = nq > 0 ? nq : 1;
  if (ozg_layout(ctx, &prm, ntiles)) return -1;
  const long nchunks = (n + OZG_ROWS - 1) / OZG_ROWS;
  long gx = ctx->num_sms / ntiles;
  if (gx < 1) gx = 1;
  if (gx > nchunks) gx = nchunks;
  const size_t pbytes = sizeof(double) * (size_t)ntiles * gx * 8192;
  char* ws = (char*)gb_workspace(ctx, pbytes + 256);
  if (!ws) return -1;
  prm.partial = (double*)ws;
  prm.err = (int*)(ws + pbytes);
  if (cudaMemsetAsync(prm.err, 0, sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "oz_gram: memset failed");
  if (cudaFuncSetAttribute(oz_gram_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, OZG_SMEM) !=
      cudaSuccess)
    return gb_fail(ctx, "oz_gram: cannot reserve %d bytes of shared memory", OZG_SMEM);
  if (tc_apply_wait_polls(ctx->opt.wait_polls, (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "oz_gram: cannot set the wait limit");
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_OZ_GRAM);
  oz_gram_kernel<<<dim3((unsigned)gx, (unsigned)ntiles), OZG_THREADS, OZG_SMEM, (cudaStream_t)ctx->stream>>>(prm);
  int rc = gb_cuda_check(ctx, (int)cudaGetLastError(), "oz_gram");
  if (rc) return rc;
  oz_gram_reduce_kernel<<<(h * wtot + 255) / 256, 256, 0, (cudaStream_t)ctx->stream>>>(
      prm.partial, (int)gx, h, nq, qoff, wtot, G, ldg, prm.err, ctx->dcount + 5);
  double bytes = (ldt == GPU_MV_FLOAT64 ? 8.0 : 4.0) * n * h;
  for (int q = 0; q < nq; q++) bytes += (prm.qdt[q] == GPU_MV_FLOAT64 ? 8.0 : 4.0) * n * prm.qw[q];
  gb_prof_end(ctx, &pr, bytes, 2.0 * n * h * wtot);
  gb_count_launch(2);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "oz_gram_reduce");
}

// ------------------------------------------------------- C-ABI entry point
extern "C" int gpu_SplitGram(gpu_MultiVector* L, gpu_MultiVector** Q, int nq, double* G_host, int ldg)
{
  gpu_Context* ctx = L->ctx;
  const int h = L->num_active;
  if (nq < 0 || nq > OZG_MAXQ) return gb_fail(ctx, "SplitGram: at most %d Q blocks", OZG_MAXQ);
  blk_cols cl;
  blk_cols* cq = (blk_cols*)malloc(sizeof(blk_cols) * (nq > 0 ? nq : 1));
  int qw[OZG_MAXQ], qdt[OZG_MAXQ];
  int wtot = h;
  if (!cq) return gb_fail(ctx, "SplitGram: out of host memory");
  gb_mv_fill_cols(L, &cl, 0);
  for (int q = 0; q < nq; q++) {
    if (Q[q]->size != L->size) {
      free(cq);
      return gb_fail(ctx, "SplitGram: block %d has %ld rows, L has %ld", q, Q[q]->size, L->size);
    }
    gb_mv_fill_cols(Q[q], &cq[q], 0);
    qw[q] = Q[q]->num_active;
    qdt[q] = Q[q]->dtype;
    wtot += qw[q];
  }
  if (ldg < h) {
    free(cq);
    return gb_fail(ctx, "SplitGram: ldg < h");
  }
  double* d = (double*)gb_device_alloc(ctx, sizeof(double) * (size_t)h * wtot);
  int rc = d ? 0 : -1;
  if (!rc) rc = gb_oz_gram(ctx, L->size, &cl, h, L->dtype, nq, cq, qw, qdt, d, h);
  double* hbuf = (double*)malloc(sizeof(double) * (size_t)h * wtot);
  if (!rc && !hbuf) rc = gb_fail(ctx, "SplitGram: out of host memory");
  if (!rc) rc = gb_memcpy_d2h(ctx, hbuf, d, sizeof(double) * (size_t)h * wtot);
  int err = 0;
  if (!rc) rc = gb_device_error(ctx, &err);
  if (!rc && err) rc = gb_fail(ctx, "SplitGram: tensor-core kernel timed out (code %d)", err);
  if (!rc)
    for (int j = 0; j < wtot; j++)
      for (int i = 0; i < h; i++) G_host[i + (size_t)j * ldg] = hbuf[i + (size_t)j * h];
  free(hbuf);
  free(cq);
  gb_sync(ctx);
  gb_device_free(d);
  return rc;
}
