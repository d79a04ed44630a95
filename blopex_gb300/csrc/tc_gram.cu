// tc_gram.cu -- the Gram matrices of one explicit-Gram LOBPCG iteration on
// the 5th-generation tensor cores:
//     G = [X R P]' [AX AR AP],   H = [X R P]' [X R P]
// for FP32 blocks of n rows and at most KP (32 or 64) columns per block,
// read from HBM once.  Replaces, for the FP32 phase of the mixed mode, the
// ten separate Gram products of the reference iteration
// (serial_Multi_VectorInnerProd via lobpcg.c:1092-1160 and the Cholesky-QR
// Grams at lobpcg.c:212).
//
// Per CTA (one per SM, a fixed slice of the rows):
//   warps 1-7  stage 32-row chunks of the six blocks into shared memory with
//              cp.async (the columns come from pointer tables: masked and
//              concatenated blocks need no copies), writing the canonical
//              128-byte-swizzled K-major layout of tcgen05 operands (each
//              block column is one 128-byte row: 32 TF32 K-elements);
//              in compensated mode they also split x = hi + lo (hi = x with
//              the low 13 mantissa bits cleared, lo = x - hi);
//   warp 0     allocates TMEM; one thread issues tcgen05.mma.kind::tf32
//              (M = 128, N = KP) into FP32 accumulators in TMEM and frees each
//              stage with tcgen05.commit; compensated mode issues
//              hi*hi + hi*lo + lo*hi;
//   warps 4-7  finally read TMEM (tcgen05.ld) and write the CTA's FP32
//              partial Gram to global memory.
// A second kernel sums the CTA partials in FP64 in a fixed order and lays
// the lower blocks out as full matrices.  CTAs cover at most
// TCG_MAX_ROWS rows so the FP32 accumulation inside TMEM stays short: it
// rounds toward zero, so a sum of positive terms (a diagonal entry) loses
// about half an ulp per MMA, ~1.5e-5 relative over 650 rows with the three
// MMAs of compensated mode; entries with mixed signs keep FP32 accuracy.
// Every wait is bounded; a timeout sets an error word and all roles finish.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "tc_common.cuh"

#define TCG_THREADS 256
#define TCG_PRODUCERS 224
#define TCG_MAX_ROWS 4096

struct tcg_params {
  blk_cols cols;  // slot s (X R P AX AR AP), column c at cols.col[s * KP + c]
  int nvalid[6];
  long n;
  long rows_per_cta;
  float* partial;  // [cta][tmem column][128 lanes]
  int* err;
};

// ------------------------------------------------------------ tile plans
// One MMA of the plan: A rows start at smem row a_row (128 rows), B rows at
// smem row b_row (N rows), accumulator at TMEM column tcol.
struct tcg_mma {
  int a_row, b_row, tcol;
};

// KP = 64: smem rows X 0-63, R 64-127, P 128-191, AX 192-255, AR 256-319,
// AP 320-383.  Lower blocks of G and H in 8 MMAs (N = 64) and 512 columns.
__constant__ tcg_mma c_plan64[8] = {{0, 192, 0},    {0, 0, 64},     {64, 256, 128}, {64, 64, 192},
                                    {128, 192, 256}, {128, 0, 320}, {128, 320, 384}, {128, 128, 448}};
// KP = 32: rows X 0-31, R 32-63, P 64-95, AX 96-127, AR 128-159, AP 160-191.
// All of G and H in 6 MMAs (N = 32) and 192 columns.
__constant__ tcg_mma c_plan32[6] = {{0, 96, 0}, {0, 128, 32}, {0, 160, 64},
                                    {0, 0, 96},  {0, 32, 128}, {0, 64, 160}};

template <int KP, int COMP>
struct tcg_cfg {
  static constexpr int ROWS = 6 * KP;               // smem rows per operand stage
  static constexpr int STAGE_BYTES = ROWS * 128;    // FP32 (or hi) tile bytes
  static constexpr int BUF_BYTES = STAGE_BYTES * (COMP ? 2 : 1);
  static constexpr int NSTAGE = (KP == 64) ? (COMP ? 2 : 4) : (COMP ? 4 : 6);
  static constexpr int NMMA = (KP == 64) ? 8 : 6;
  static constexpr int TMEM_COLS = (KP == 64) ? 512 : 256;
  static constexpr int USED_COLS = (KP == 64) ? 512 : 192;
  static constexpr int LAG = NSTAGE > 2 ? NSTAGE - 2 : 1;  // cp.async groups kept in flight
};

template <int KP, int COMP>
__global__ void __launch_bounds__(TCG_THREADS, 1) tc_gram_kernel(const __grid_constant__ tcg_params prm)
{
  using C = tcg_cfg<KP, COMP>;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte aligned operand stages (SW128 atoms)
  unsigned char* smem = smem_align1024(smem_raw);
  __shared__ uint64_t full_bar[C::NSTAGE], empty_bar[C::NSTAGE], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const long r_begin = (long)blockIdx.x * prm.rows_per_cta;
  const long r_end = min(prm.n, r_begin + prm.rows_per_cta);
  const int nchunks = (int)((r_end - r_begin + 31) / 32);

  if (tid == 0) {
    abort_flag = 0;
    for (int s = 0; s < C::NSTAGE; s++) {
      mbar_init(&full_bar[s], TCG_PRODUCERS);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&done_bar, 1);
  }
  // zero every stage once: rows of absent columns stay zero
  for (int e = tid; e < C::NSTAGE * C::BUF_BYTES / 16; e += TCG_THREADS)
    ((uint4*)smem)[e] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base)),
                 "r"((uint32_t)C::TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_proxy_async();
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmem_base;

  if (warp >= 1) {
    // ---------------------------------------------------------- producers
    const int p = tid - 32;
    const int units = C::ROWS * 8;  // 16-byte pieces per stage
    int pending = 0;                // chunks issued but not yet released
    for (int c = 0; c < nchunks && !abort_flag; c++) {
      const int s = c % C::NSTAGE;
      if (c >= C::NSTAGE && !mbar_wait(&empty_bar[s], ((c / C::NSTAGE) - 1) & 1, &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 1);
        break;
      }
      unsigned char* st = smem + (size_t)s * C::BUF_BYTES;
      const long row0 = r_begin + (long)c * 32;
      for (int u = p; u < units; u += TCG_PRODUCERS) {
        const int row = u >> 3, q = u & 7;
        const int slot = row / KP, col = row % KP;
        if (col >= prm.nvalid[slot]) continue;
        const long r = row0 + 4 * q;
        long left = (r_end - r) * 4;
        const uint32_t bytes = left >= 16 ? 16u : (left > 0 ? (uint32_t)left : 0u);
        const float* src = (const float*)prm.cols.col[slot * KP + col] + (bytes ? r : 0);
        cp_async16(smem_u32(st + row * 128 + ((q ^ (row & 7)) << 4)), src, bytes);
      }
      cp_async_commit();
      pending++;
      if (pending > C::LAG) {
        cp_async_wait<C::LAG>();
        const int cr = c - C::LAG;  // oldest chunk: its copies have landed
        unsigned char* sr = smem + (size_t)(cr % C::NSTAGE) * C::BUF_BYTES;
        if (COMP) {
          for (int u = p; u < units; u += TCG_PRODUCERS) {
            const int row = u >> 3, q = u & 7;
            uint32_t off = row * 128 + ((q ^ (row & 7)) << 4);
            float4 v = *(float4*)(sr + off);
            float4 h, l;
            h.x = __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u);
            h.y = __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u);
            h.z = __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u);
            h.w = __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u);
            l.x = v.x - h.x;
            l.y = v.y - h.y;
            l.z = v.z - h.z;
            l.w = v.w - h.w;
            *(float4*)(sr + off) = h;
            *(float4*)(sr + C::STAGE_BYTES + off) = l;
          }
        }
        fence_proxy_async();
        mbar_arrive(&full_bar[cr % C::NSTAGE]);
        pending--;
      }
    }
    // drain
    cp_async_wait<0>();
    for (int c = nchunks - pending; c < nchunks && pending > 0 && !abort_flag; c++) {
      unsigned char* sr = smem + (size_t)(c % C::NSTAGE) * C::BUF_BYTES;
      if (COMP) {
        for (int u = p; u < units; u += TCG_PRODUCERS) {
          const int row = u >> 3, q = u & 7;
          uint32_t off = row * 128 + ((q ^ (row & 7)) << 4);
          float4 v = *(float4*)(sr + off);
          float4 h, l;
          h.x = __uint_as_float(__float_as_uint(v.x) & 0xFFFFE000u);
          h.y = __uint_as_float(__float_as_uint(v.y) & 0xFFFFE000u);
          h.z = __uint_as_float(__float_as_uint(v.z) & 0xFFFFE000u);
          h.w = __uint_as_float(__float_as_uint(v.w) & 0xFFFFE000u);
          l.x = v.x - h.x;
          l.y = v.y - h.y;
          l.z = v.z - h.z;
          l.w = v.w - h.w;
          *(float4*)(sr + off) = h;
          *(float4*)(sr + C::STAGE_BYTES + off) = l;
        }
      }
      fence_proxy_async();
      mbar_arrive(&full_bar[c % C::NSTAGE]);
    }
  } else if (lane == 0) {
    // ----------------------------------------------------------- MMA issuer
    const uint32_t idesc = tf32_idesc(128, KP);
    for (int c = 0; c < nchunks; c++) {
      const int s = c % C::NSTAGE;
      if (!mbar_wait(&full_bar[s], (c / C::NSTAGE) & 1, &abort_flag)) {
        abort_flag = 1;
        atomicExch(prm.err, 2);
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t base = smem_u32(smem + (size_t)s * C::BUF_BYTES);
      for (int kk = 0; kk < 4; kk++) {  // 4 x K=8 TF32 steps across the 128-byte row
        for (int e = 0; e < C::NMMA; e++) {
          const tcg_mma mm = (KP == 64) ? c_plan64[e] : c_plan32[e];
          const uint32_t a = base + mm.a_row * 128 + kk * 32;
          const uint32_t b = base + mm.b_row * 128 + kk * 32;
          const uint32_t d = tmem + mm.tcol;
          const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(d, sw128_desc(a), sw128_desc(b), idesc, acc);
          if (COMP) {
            mma_tf32(d, sw128_desc(a), sw128_desc(b + C::STAGE_BYTES), idesc, 1u);
            mma_tf32(d, sw128_desc(a + C::STAGE_BYTES), sw128_desc(b), idesc, 1u);
          }
        }
      }
      mma_commit(&empty_bar[s]);  // the stage is free once these MMAs finish
    }
    mma_commit(&done_bar);
  }

  // ------------------------------------------------------------ epilogue
  if (warp >= 4) {
    // the issuer always commits done_bar after its last MMA, so this wait
    // also guarantees no MMA is in flight when TMEM is read and freed
    const bool ok = mbar_drain(&done_bar, 0) && !abort_flag;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int quarter = warp - 4;  // TMEM lanes 32*quarter .. +31
    float* out = prm.partial + (size_t)blockIdx.x * C::USED_COLS * 128;
    for (int g = 0; g < C::USED_COLS / 32; g++) {
      uint32_t r[32];
      const uint32_t taddr = tmem + ((uint32_t)(32 * quarter) << 16) + (uint32_t)(g * 32);
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
          "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
            "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
            "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
            "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
            "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
            "=r"(r[31])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      const int ln = 32 * quarter + lane;
#pragma unroll
      for (int j = 0; j < 32; j++)
        out[(size_t)(g * 32 + j) * 128 + ln] = ok ? __uint_as_float(r[j]) : 0.f;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"((uint32_t)C::TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------- reduction
// padded index of compact index i for blocks of sizes (k, nR, nP) in slots of KP
__device__ __forceinline__ int tcg_pad(int i, int k, int nR, int KP)
{
  if (i < k) return i;
  if (i < k + nR) return KP + (i - k);
  return 2 * KP + (i - k - nR);
}

// TMEM (column, lane) holding entry (left pi, right pj) of G (which = 0) or H
// (which = 1), -1 if that block is not computed (the transposed one is)
__device__ __forceinline__ int tcg_locate(int which, int pi, int pj, int KP, int* lane)
{
  if (KP == 32) {
    *lane = pi;
    return which * 96 + pj;
  }
  const int rb = pj / 64;
  if (rb == 0) {
    if (pi < 128) {
      *lane = pi;
      return (which ? 64 : 0) + pj;
    }
    *lane = pi - 128;
    return (which ? 320 : 256) + pj;
  }
  if (rb == 1) {
    if (pi < 64) return -1;
    *lane = pi - 64;
    return (which ? 192 : 128) + (pj - 64);
  }
  if (pi < 128) return -1;
  *lane = pi - 128;
  return (which ? 448 : 384) + (pj - 128);
}

__global__ void tc_gram_reduce_kernel(const float* __restrict__ partial, int nctas, int used_cols,
                                      int KP, int k, int nR, int nP, double* G, double* H, int ld,
                                      const int* err, int* status)
{
  // a timed-out wait is also reported through the context's device error word
  if (blockIdx.x == 0 && threadIdx.x == 0 && *err) *status = *err;
  const int m = k + nR + nP;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 2 * m * m) return;
  const int which = e / (m * m);
  const int i = (e % (m * m)) % m, j = (e % (m * m)) / m;
  int pi = tcg_pad(i, k, nR, KP), pj = tcg_pad(j, k, nR, KP);
  int lane;
  int col = tcg_locate(which, pi, pj, KP, &lane);
  if (col < 0) col = tcg_locate(which, pj, pi, KP, &lane);
  double sum = 0.0;
  for (int c = 0; c < nctas; c++) sum += (double)partial[((size_t)c * used_cols + col) * 128 + lane];
  if (*err) sum = __longlong_as_double(0x7ff8000000000000LL);  // NaN: the caller sees a failed Gram
  (which ? H : G)[i + (size_t)j * ld] = sum;
}

// ------------------------------------------------------------------- host
template <int KP, int COMP>
static int tc_launch(gpu_Context* ctx, long n, tcg_params* prm, int nctas)
{
  using C = tcg_cfg<KP, COMP>;
  const size_t smem = (size_t)C::NSTAGE * C::BUF_BYTES + 1024;
  if (cudaFuncSetAttribute(tc_gram_kernel<KP, COMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return gb_fail(ctx, "tc_gram: cannot reserve %zu bytes of shared memory", smem);
  if (tc_apply_wait_polls(ctx->opt.wait_polls, (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "tc_gram: cannot set the wait limit");
  tc_gram_kernel<KP, COMP><<<nctas, TCG_THREADS, smem, (cudaStream_t)ctx->stream>>>(*prm);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "tc_gram");
}

extern "C" int gb_tc_gram(gpu_Context* ctx, long n, const blk_cols* X, int k, const blk_cols* R,
                          int nR, const blk_cols* P, int nP, const blk_cols* AX,
                          const blk_cols* AR, const blk_cols* AP, int compensated, double* G,
                          double* H, int ld)
{
  const int KP = k <= 32 ? 32 : 64;
  if (k > 64 || nR > KP || nP > KP || n <= 0)
    return gb_fail(ctx, "tc_gram: block widths (%d, %d, %d) not supported", k, nR, nP);
  tcg_params prm;
  memset(&prm, 0, sizeof(prm));
  const blk_cols* src[6] = {X, R, P, AX, AR, AP};
  const int cnt[6] = {k, nR, nP, k, nR, nP};
  for (int s = 0; s < 6; s++) {
    prm.nvalid[s] = cnt[s];
    for (int c = 0; c < cnt[s]; c++) {
      prm.cols.col[s * KP + c] = src[s]->col[c];
      // the producers copy 16-byte pieces: every column must start on 16 bytes
      if ((uintptr_t)src[s]->col[c] & 15)
        return gb_fail(ctx, "tc_gram: column %d of block %d not 16-byte aligned", c, s);
    }
  }
  // CTAs: whole waves of the SMs, each with at most TCG_MAX_ROWS rows
  long waves = (n + (long)ctx->num_sms * TCG_MAX_ROWS - 1) / ((long)ctx->num_sms * TCG_MAX_ROWS);
  if (waves < 1) waves = 1;
  long nctas = waves * ctx->num_sms;
  long rows = (n + nctas - 1) / nctas;
  rows = (rows + 31) / 32 * 32;
  nctas = (n + rows - 1) / rows;
  const int used = KP == 64 ? 512 : 192;
  const size_t pbytes = sizeof(float) * (size_t)nctas * used * 128;
  char* ws = (char*)gb_workspace(ctx, pbytes + 256);
  if (!ws) return -1;
  prm.partial = (float*)ws;
  prm.err = (int*)(ws + pbytes);
  prm.n = n;
  prm.rows_per_cta = rows;
  if (cudaMemsetAsync(prm.err, 0, sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess)
    return gb_fail(ctx, "tc_gram: memset failed");
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_TC_GRAM);
  int rc;
  if (KP == 64)
    rc = compensated ? tc_launch<64, 1>(ctx, n, &prm, (int)nctas) : tc_launch<64, 0>(ctx, n, &prm, (int)nctas);
  else
    rc = compensated ? tc_launch<32, 1>(ctx, n, &prm, (int)nctas) : tc_launch<32, 0>(ctx, n, &prm, (int)nctas);
  if (rc) return rc;
  const int m = k + nR + nP;
  tc_gram_reduce_kernel<<<(2 * m * m + 255) / 256, 256, 0, (cudaStream_t)ctx->stream>>>(
      prm.partial, (int)nctas, used, KP, k, nR, nP, G, H, ld, prm.err, ctx->dcount + 5);
  const double bytes = 4.0 * n * 2.0 * (k + nR + nP);
  const double flops = 2.0 * 2.0 * n * (double)m * m * (compensated ? 3.0 : 1.0);
  gb_prof_end(ctx, &pr, bytes, flops);
  gb_count_launch(2);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "tc_gram_reduce");
}

// ------------------------------------------------------- C-ABI entry point
extern "C" int gpu_ExplicitGram(gpu_MultiVector* X, gpu_MultiVector* R, gpu_MultiVector* P,
                                gpu_MultiVector* AX, gpu_MultiVector* AR, gpu_MultiVector* AP,
                                int mode, double* G_host, double* H_host, int ldh)
{
  gpu_Context* ctx = X->ctx;
  const int k = X->num_active, nR = R ? R->num_active : 0, nP = P ? P->num_active : 0;
  const int m = k + nR + nP;
  if (ldh < m) return gb_fail(ctx, "ExplicitGram: ldh < m");
  if (mode != 0 && X->dtype != GPU_MV_FLOAT32) return gb_fail(ctx, "ExplicitGram: tensor modes need FP32 blocks");
  blk_cols cx, cr, cp, cax, car, cap;
  gb_mv_fill_cols(X, &cx, 0);
  gb_mv_fill_cols(AX, &cax, 0);
  if (R) {
    gb_mv_fill_cols(R, &cr, 0);
    gb_mv_fill_cols(AR, &car, 0);
  }
  if (P) {
    gb_mv_fill_cols(P, &cp, 0);
    gb_mv_fill_cols(AP, &cap, 0);
  }
  double* d = (double*)gb_device_alloc(ctx, sizeof(double) * 2 * (size_t)m * m);
  if (!d) return -1;
  int rc;
  if (mode == 0) {
    blk_cols left, right, rightb;
    int off = gb_mv_fill_cols(X, &left, 0);
    if (R) off = gb_mv_fill_cols(R, &left, off);
    if (P) gb_mv_fill_cols(P, &left, off);
    off = gb_mv_fill_cols(AX, &right, 0);
    if (R) off = gb_mv_fill_cols(AR, &right, off);
    if (P) gb_mv_fill_cols(AP, &right, off);
    rightb = left;
    rc = gb_gram(ctx, X->dtype, X->size, &left, m, &right, m, d, m);
    if (!rc) rc = gb_gram(ctx, X->dtype, X->size, &left, m, &rightb, m, d + (size_t)m * m, m);
  } else {
    rc = gb_tc_gram(ctx, X->size, &cx, k, &cr, nR, &cp, nP, &cax, &car, &cap, mode == 2, d,
                    d + (size_t)m * m, m);
  }
  double* h = (double*)malloc(sizeof(double) * 2 * (size_t)m * m);
  if (!rc) rc = gb_memcpy_d2h(ctx, h, d, sizeof(double) * 2 * (size_t)m * m);
  if (!rc)
    for (int j = 0; j < m; j++)
      for (int i = 0; i < m; i++) {
        G_host[i + (size_t)j * ldh] = h[i + (size_t)j * m];
        H_host[i + (size_t)j * ldh] = h[(size_t)m * m + i + (size_t)j * m];
      }
  free(h);
  gb_device_free(d);
  return rc;
}
