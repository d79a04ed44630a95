// blockops.cu -- tall-skinny block kernels on column-major multivectors
// (CUDA-core versions, FP64 and FP32 storage):
//   Gram        G = X' Y          (serial_Multi_VectorInnerProd, multi_vector.c:354-406);
//               X' X of one block on the lower triangle only, bit-identical
//   X*C update  Y = X C [+ Z]     (serial_Multi_VectorByMatrix, multi_vector.c:474-524);
//               C upper triangular: the zero triangle skipped, bit-identical
//   axpby, column scaling, column dots, residual, precision conversion,
//   drand48 fill (multi_vector.c:165-184).
// Columns are addressed through blk_cols pointer tables, so masked
// (non-contiguous) columns and concatenated blocks [X R P] cost nothing.
// Split-k partial sums are reduced in a fixed order: results are
// deterministic run to run.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "internal.h"
#include "blas32.cuh"

#define CUDA_LAUNCH_CHECK(ctx, what) gb_cuda_check((ctx), (int)cudaGetLastError(), (what))

static inline cudaStream_t S(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

// ------------------------------------------------------------------------
// Gram: partial[s][j*h + i] = sum over rows of split s of X(r,i) * Y(r,j)
// 256 threads as 16 x 16; each thread owns a TM x TN register tile with
// rows ty + 16*a and columns tx + 16*b; rows are staged 32 at a time.
// FP32 inputs accumulate in FP32 over 128-row blocks, flushed to FP64.
// ------------------------------------------------------------------------
template <typename T, int TM, int TN>
__global__ void __launch_bounds__(256) gram_partial_kernel(blk_cols X, int h, blk_cols Y, int w,
                                                           long n, long rows_per_split,
                                                           double* __restrict__ partial)
{
  constexpr int BM = 16 * TM, BN = 16 * TN, RK = 32;
  __shared__ T xs[RK][BM + 1];
  __shared__ T ys[RK][BN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * BM, j0 = blockIdx.y * BN;
  const long r_begin = (long)blockIdx.z * rows_per_split;
  const long r_end = min(n, r_begin + rows_per_split);

  double acc[TM][TN];
  T accs[TM][TN];
#pragma unroll
  for (int a = 0; a < TM; a++)
#pragma unroll
    for (int b = 0; b < TN; b++) {
      acc[a][b] = 0.0;
      accs[a][b] = T(0);
    }

  int chunk = 0;
  for (long r0 = r_begin; r0 < r_end; r0 += RK) {
    // stage rows r0..r0+RK of the BM columns of X and BN columns of Y
    for (int e = threadIdx.x; e < RK * BM; e += 256) {
      int rr = e % RK, cc = e / RK;
      long r = r0 + rr;
      int c = i0 + cc;
      T v = T(0);
      if (r < r_end && c < h) v = ((const T*)X.col[c])[r];
      xs[rr][cc] = v;
    }
    for (int e = threadIdx.x; e < RK * BN; e += 256) {
      int rr = e % RK, cc = e / RK;
      long r = r0 + rr;
      int c = j0 + cc;
      T v = T(0);
      if (r < r_end && c < w) v = ((const T*)Y.col[c])[r];
      ys[rr][cc] = v;
    }
    __syncthreads();
#pragma unroll 8
    for (int rr = 0; rr < RK; rr++) {
      T xv[TM], yv[TN];
#pragma unroll
      for (int a = 0; a < TM; a++) xv[a] = xs[rr][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < TN; b++) yv[b] = ys[rr][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < TM; a++)
#pragma unroll
        for (int b = 0; b < TN; b++) accs[a][b] = fma(xv[a], yv[b], accs[a][b]);
    }
    __syncthreads();
    if (sizeof(T) == 8 || (++chunk & 3) == 0) {
#pragma unroll
      for (int a = 0; a < TM; a++)
#pragma unroll
        for (int b = 0; b < TN; b++) {
          acc[a][b] += (double)accs[a][b];
          accs[a][b] = T(0);
        }
    }
  }
  double* out = partial + (size_t)blockIdx.z * h * w;
#pragma unroll
  for (int a = 0; a < TM; a++)
#pragma unroll
    for (int b = 0; b < TN; b++) {
      int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < h && j < w) out[(size_t)j * h + i] = acc[a][b] + (double)accs[a][b];
    }
}

__global__ void gram_reduce_kernel(const double* __restrict__ partial, int splits, int h, int w,
                                   double* __restrict__ G, int ldg)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= h * w) return;
  double s = 0.0;
  for (int p = 0; p < splits; p++) s += partial[(size_t)p * h * w + e];
  int i = e % h, j = e / h;
  G[(size_t)j * ldg + i] = s;
}

// Symmetric Gram X'X (h <= 64) on the lower triangle only.  Thread t owns
// the BS x BS block (bi, bj), bi >= bj, of the triangular numbering t =
// bi (bi + 1) / 2 + bj, so whole warps drop out of the upper triangle (a
// warp-wide FP64 instruction costs the same whatever its lane count).  Row
// splits, staging, the order of the multiply-adds into each entry and the
// flushes to FP64 are those of gram_partial_kernel, so every entry (and its
// mirror, as x_i x_j = x_j x_i exactly) is bit-identical to the full
// product's.
template <typename T, int BS>
__global__ void __launch_bounds__(544) gram_sym_partial_kernel(blk_cols X, int h, long n,
                                                               long rows_per_split,
                                                               double* __restrict__ partial)
{
  constexpr int BM = 32 * BS, RK = 32;
  __shared__ T xs[RK][BM + 1];
  const int t = threadIdx.x;
  const int nb = (h + BS - 1) / BS;
  const bool active = t < nb * (nb + 1) / 2;
  int bi = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  while (bi * (bi + 1) / 2 > t) bi--;
  while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
  const int bj = t - bi * (bi + 1) / 2;
  const long r_begin = (long)blockIdx.z * rows_per_split;
  const long r_end = min(n, r_begin + rows_per_split);

  double acc[BS][BS];
  T accs[BS][BS];
#pragma unroll
  for (int a = 0; a < BS; a++)
#pragma unroll
    for (int b = 0; b < BS; b++) {
      acc[a][b] = 0.0;
      accs[a][b] = T(0);
    }

  int chunk = 0;
  for (long r0 = r_begin; r0 < r_end; r0 += RK) {
    for (int e = t; e < RK * BM; e += blockDim.x) {
      int rr = e % RK, cc = e / RK;
      long r = r0 + rr;
      T v = T(0);
      if (r < r_end && cc < h) v = ((const T*)X.col[cc])[r];
      xs[rr][cc] = v;
    }
    __syncthreads();
    if (active) {
#pragma unroll 8
      for (int rr = 0; rr < RK; rr++) {
        T xv[BS], yv[BS];
#pragma unroll
        for (int a = 0; a < BS; a++) xv[a] = xs[rr][BS * bi + a];
#pragma unroll
        for (int b = 0; b < BS; b++) yv[b] = xs[rr][BS * bj + b];
#pragma unroll
        for (int a = 0; a < BS; a++)
#pragma unroll
          for (int b = 0; b < BS; b++) accs[a][b] = fma(xv[a], yv[b], accs[a][b]);
      }
    }
    __syncthreads();
    if (sizeof(T) == 8 || (++chunk & 3) == 0) {
#pragma unroll
      for (int a = 0; a < BS; a++)
#pragma unroll
        for (int b = 0; b < BS; b++) {
          acc[a][b] += (double)accs[a][b];
          accs[a][b] = T(0);
        }
    }
  }
  if (!active) return;
  double* out = partial + (size_t)blockIdx.z * h * h;
#pragma unroll
  for (int a = 0; a < BS; a++)
#pragma unroll
    for (int b = 0; b < BS; b++) {
      const int i = BS * bi + a, j = BS * bj + b;
      if (i < h && j <= i) out[(size_t)j * h + i] = acc[a][b] + (double)accs[a][b];
    }
}

// G (h x h) from the lower-triangle partials, both triangles
__global__ void gram_sym_reduce_kernel(const double* __restrict__ partial, int splits, int h,
                                       double* __restrict__ G, int ldg)
{
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= h * h) return;
  int i = e % h, j = e / h;
  const int src = i >= j ? e : j + i * h;
  double s = 0.0;
  for (int p = 0; p < splits; p++) s += partial[(size_t)p * h * h + src];
  G[(size_t)j * ldg + i] = s;
}

// the row splits of gram_launch for a single (gx = gy = 1) output tile
static long gram_splits(gpu_Context* ctx, long n, long* rows)
{
  long splits = 2 * ctx->num_sms;
  long max_splits = (n + 255) / 256;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  long r = (n + splits - 1) / splits;
  r = (r + 31) / 32 * 32;
  splits = (n + r - 1) / r;
  if (splits < 1) splits = 1;
  *rows = r;
  return splits;
}

template <typename T, int BS>
static int gram_sym_launch(gpu_Context* ctx, long n, const blk_cols* X, int h, double* G, int ldg)
{
  long rows;
  const long splits = gram_splits(ctx, n, &rows);
  double* partial = (double*)gb_workspace(ctx, sizeof(double) * (size_t)splits * h * h);
  if (!partial) return -1;
  const int nb = (h + BS - 1) / BS;
  const int threads = (nb * (nb + 1) / 2 + 31) / 32 * 32;
  dim3 grid(1, 1, (unsigned)splits);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, sizeof(T) == 8 ? GB_K_GRAM : GB_K_GRAM32);
  gram_sym_partial_kernel<T, BS><<<grid, threads, 0, S(ctx)>>>(*X, h, n, rows, partial);
  gram_sym_reduce_kernel<<<(h * h + 255) / 256, 256, 0, S(ctx)>>>(partial, (int)splits, h, G, ldg);
  gb_prof_end(ctx, &pr, (double)sizeof(T) * n * h, (double)n * h * (h + 1));
  gb_count_launch(2);
  return CUDA_LAUNCH_CHECK(ctx, "gram_sym");
}

template <typename T, int TM, int TN>
static int gram_launch(gpu_Context* ctx, long n, const blk_cols* X, int h, const blk_cols* Y,
                       int w, double* G, int ldg)
{
  constexpr int BM = 16 * TM, BN = 16 * TN;
  int gx = (h + BM - 1) / BM, gy = (w + BN - 1) / BN;
  int target = 2 * ctx->num_sms;
  long splits = target / (gx * gy);
  if (splits < 1) splits = 1;
  long max_splits = (n + 255) / 256;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  long rows = (n + splits - 1) / splits;
  rows = (rows + 31) / 32 * 32;
  splits = (n + rows - 1) / rows;
  if (splits < 1) splits = 1;
  double* partial = (double*)gb_workspace(ctx, sizeof(double) * (size_t)splits * h * w);
  if (!partial) return -1;
  dim3 grid(gx, gy, (unsigned)splits);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, sizeof(T) == 8 ? GB_K_GRAM : GB_K_GRAM32);
  gram_partial_kernel<T, TM, TN><<<grid, 256, 0, S(ctx)>>>(*X, h, *Y, w, n, rows, partial);
  int tot = h * w;
  gram_reduce_kernel<<<(tot + 255) / 256, 256, 0, S(ctx)>>>(partial, (int)splits, h, w, G, ldg);
  gb_prof_end(ctx, &pr, (double)sizeof(T) * n * (h + w), 2.0 * n * h * w);
  gb_count_launch(2);
  return CUDA_LAUNCH_CHECK(ctx, "gram");
}

extern "C" int gb_gram(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h,
                       const blk_cols* Y, int w, double* G, int ldg)
{
  if (h <= 0 || w <= 0) return 0;
  // X'X with h <= 64 (one output tile): the lower triangle only
  if (h == w && h <= 64 && memcmp(X->col, Y->col, sizeof(void*) * (size_t)h) == 0) {
    if (dtype == GPU_MV_FLOAT64)
      return h <= 32 ? gram_sym_launch<double, 1>(ctx, n, X, h, G, ldg)
                     : gram_sym_launch<double, 2>(ctx, n, X, h, G, ldg);
    return h <= 32 ? gram_sym_launch<float, 1>(ctx, n, X, h, G, ldg)
                   : gram_sym_launch<float, 2>(ctx, n, X, h, G, ldg);
  }
  if (dtype == GPU_MV_FLOAT64) {
    if (h <= 32 && w <= 32) return gram_launch<double, 2, 2>(ctx, n, X, h, Y, w, G, ldg);
    return gram_launch<double, 4, 4>(ctx, n, X, h, Y, w, G, ldg);
  }
  if (h <= 32 && w <= 32) return gram_launch<float, 2, 2>(ctx, n, X, h, Y, w, G, ldg);
  return gram_launch<float, 4, 4>(ctx, n, X, h, Y, w, G, ldg);
}

// ------------------------------------------------------------------------
// X*C update: Y(:, j0:j0+32) for 64 rows per CTA; thread t owns row t%64
// and 8 columns (t/64)*8 ... ; K staged 32 at a time in shared memory.
// tri: C is upper triangular with explicit zeros below the diagonal (a
// Cholesky-QR factor); a warp stops at its last column's diagonal, skipping
// only terms that add an exact zero, so Y is bit-identical to the full
// product.
// ------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) bymat_kernel(blk_cols X, int h, const double* __restrict__ C,
                                                    int ldc, blk_cols Y, int w, blk_cols Z,
                                                    int has_z, long n, int tri)
{
  constexpr int BM = 64, BN = 32, KC = 32;
  __shared__ T xs[KC][BM];
  __shared__ T cs[KC][BN];
  const int t = threadIdx.x;
  const int rl = t & 63, cg = t >> 6;
  const long r0 = (long)blockIdx.x * BM;
  const int j0 = blockIdx.y * BN;
  T acc[8];
#pragma unroll
  for (int b = 0; b < 8; b++) acc[b] = T(0);

  const int kmax = tri ? min(h, j0 + BN) : h;
  for (int k0 = 0; k0 < kmax; k0 += KC) {
    for (int e = t; e < KC * BM; e += 256) {
      int rr = e % BM, kk = e / BM;
      long r = r0 + rr;
      T v = T(0);
      if (r < n && k0 + kk < h) v = ((const T*)X.col[k0 + kk])[r];
      xs[kk][rr] = v;
    }
    for (int e = t; e < KC * BN; e += 256) {
      int kk = e % KC, jj = e / KC;
      T v = T(0);
      if (k0 + kk < h && j0 + jj < w) v = (T)C[(size_t)(j0 + jj) * ldc + k0 + kk];
      cs[kk][jj] = v;
    }
    __syncthreads();
    const int kk_end = tri ? max(0, min(KC, j0 + cg * 8 + 8 - k0)) : KC;
#pragma unroll 8
    for (int kk = 0; kk < kk_end; kk++) {
      T xv = xs[kk][rl];
#pragma unroll
      for (int b = 0; b < 8; b++) acc[b] = fma(xv, cs[kk][cg * 8 + b], acc[b]);
    }
    __syncthreads();
  }
  long r = r0 + rl;
  if (r < n) {
#pragma unroll
    for (int b = 0; b < 8; b++) {
      int j = j0 + cg * 8 + b;
      if (j < w) {
        T v = acc[b];
        if (has_z) v += ((const T*)Z.col[j])[r];
        ((T*)Y.col[j])[r] = v;
      }
    }
  }
}

static int bymat_launch(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h,
                        const double* C, int ldc, const blk_cols* Y, int w, const blk_cols* Z,
                        int tri)
{
  if (w <= 0 || n <= 0) return 0;
  dim3 grid((unsigned)((n + 63) / 64), (w + 31) / 32);
  blk_cols empty;
  const blk_cols* z = Z ? Z : &empty;
  const double es = dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0;
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, dtype == GPU_MV_FLOAT64 ? GB_K_XC : GB_K_XC32);
  if (dtype == GPU_MV_FLOAT64)
    bymat_kernel<double><<<grid, 256, 0, S(ctx)>>>(*X, h, C, ldc, *Y, w, *z, Z != NULL, n, tri);
  else
    bymat_kernel<float><<<grid, 256, 0, S(ctx)>>>(*X, h, C, ldc, *Y, w, *z, Z != NULL, n, tri);
  // a triangular C: sum over j of min(j + 1, h) products per row
  const double kw = tri ? (double)w * (w + 1) / 2 - (w > h ? (double)(w - h) * (w - h + 1) / 2 : 0.0)
                        : (double)h * w;
  gb_prof_end(ctx, &pr, es * n * (h + w + (Z ? w : 0)), 2.0 * n * kw);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "bymat");
}

extern "C" int gb_bymat(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h,
                        const double* C, int ldc, const blk_cols* Y, int w, const blk_cols* Z)
{
  return bymat_launch(ctx, dtype, n, X, h, C, ldc, Y, w, Z, 0);
}

extern "C" int gb_bymat_tri(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h,
                            const double* C, int ldc, const blk_cols* Y, int w)
{
  return bymat_launch(ctx, dtype, n, X, h, C, ldc, Y, w, NULL, 1);
}

// ------------------------------------------------------------------------
// elementwise column kernels: grid.y = column, grid-stride over rows
// ------------------------------------------------------------------------
template <typename T>
__global__ void axpby_kernel(blk_cols X, double alpha, blk_cols Y, double beta, long n)
{
  const T* x = (const T*)X.col[blockIdx.y];
  T* y = (T*)Y.col[blockIdx.y];
  const T a = (T)alpha, b = (T)beta;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    if (beta == 0.0)
      y[r] = a * x[r];
    else
      y[r] = a * x[r] + b * y[r];
  }
}

static unsigned row_blocks(gpu_Context* ctx, long n, int w)
{
  long want = (n + 255) / 256;
  long cap = (long)ctx->num_sms * 8 / (w > 0 ? w : 1);
  if (cap < 4) cap = 4;
  if (want > cap) want = cap;
  if (want < 1) want = 1;
  return (unsigned)want;
}

extern "C" int gb_axpby(gpu_Context* ctx, int dtype, long n, double alpha, const blk_cols* X,
                        double beta, const blk_cols* Y, int w)
{
  if (w <= 0 || n <= 0) return 0;
  dim3 grid(row_blocks(ctx, n, w), w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  if (dtype == GPU_MV_FLOAT64)
    axpby_kernel<double><<<grid, 256, 0, S(ctx)>>>(*X, alpha, *Y, beta, n);
  else
    axpby_kernel<float><<<grid, 256, 0, S(ctx)>>>(*X, alpha, *Y, beta, n);
  gb_prof_end(ctx, &pr, (dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0) * n * w * (beta == 0.0 ? 2 : 3), 0.0);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "axpby");
}

struct idx_table {
  int v[BLK_MAXCOLS];
};

template <typename T>
__global__ void scale_cols_kernel(blk_cols X, const double* __restrict__ d, idx_table idx,
                                  blk_cols Y, long n)
{
  const T* x = (const T*)X.col[blockIdx.y];
  T* y = (T*)Y.col[blockIdx.y];
  const T a = (T)d[idx.v[blockIdx.y]];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    y[r] = a * x[r];
}

static void fill_idx(idx_table* t, const int* idx, int w)
{
  for (int j = 0; j < w; j++) t->v[j] = idx ? idx[j] : j;
}

extern "C" int gb_scale_cols(gpu_Context* ctx, int dtype, long n, const blk_cols* X,
                             const double* d, const int* idx, const blk_cols* Y, int w)
{
  if (w <= 0 || n <= 0) return 0;
  idx_table t;
  fill_idx(&t, idx, w);
  dim3 grid(row_blocks(ctx, n, w), w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  if (dtype == GPU_MV_FLOAT64)
    scale_cols_kernel<double><<<grid, 256, 0, S(ctx)>>>(*X, d, t, *Y, n);
  else
    scale_cols_kernel<float><<<grid, 256, 0, S(ctx)>>>(*X, d, t, *Y, n);
  gb_prof_end(ctx, &pr, (dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0) * n * w * 2, 0.0);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "scale_cols");
}

// column dot products: per-CTA partial sums, then a fixed-order reduction
template <typename T>
__global__ void dot_partial_kernel(blk_cols X, blk_cols Y, long n, double* __restrict__ partial)
{
  const T* x = (const T*)X.col[blockIdx.y];
  const T* y = (const T*)Y.col[blockIdx.y];
  double s = 0.0;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    s += (double)x[r] * (double)y[r];
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

__global__ void dot_reduce_kernel(const double* __restrict__ partial, int nb, idx_table idx,
                                  int w, double* __restrict__ out)
{
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= w) return;
  double s = 0.0;
  for (int b = 0; b < nb; b++) s += partial[(size_t)j * nb + b];
  out[idx.v[j]] = s;
}

// FP32 blocks with 16-byte aligned columns: float4 loads, exact products in
// a compensated FP32 sum flushed to FP64 every 64 terms (blas32.cuh)
__global__ void __launch_bounds__(256) dot32_partial_kernel(blk_cols X, blk_cols Y, long n,
                                                            double* __restrict__ partial)
{
  const float4* x = (const float4*)X.col[blockIdx.y];
  const float4* y = (const float4*)Y.col[blockIdx.y];
  const long n4 = n >> 2, stride = (long)gridDim.x * blockDim.x;
  double acc = 0.0;
  float s = 0.f, c = 0.f;
  int cnt = 0;
#pragma unroll 4
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < n4; v += stride) {
    acc_prod32x4(s, c, x[v], y[v]);
    if (++cnt == 16) {
      acc += (double)s + (double)c;
      s = c = 0.f;
      cnt = 0;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {  // the last n % 4 rows
    const long r = 4 * n4 + threadIdx.x;
    acc_prod32(s, c, ((const float*)x)[r], ((const float*)y)[r]);
  }
  acc += (double)s + (double)c;
  const double t = block_sum256(acc);
  if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
}

extern "C" int gb_dot_reduce(gpu_Context* ctx, const double* partial, int nb, int w, double* out,
                             const int* idx)
{
  idx_table t;
  fill_idx(&t, idx, w);
  dot_reduce_kernel<<<(w + 63) / 64, 64, 0, S(ctx)>>>(partial, nb, t, w, out);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "dot_reduce");
}

extern "C" unsigned gb_row_blocks(gpu_Context* ctx, long n, int w) { return row_blocks(ctx, n, w); }

extern "C" int gb_dot_cols(gpu_Context* ctx, int dtype, long n, const blk_cols* X,
                           const blk_cols* Y, int w, double* out, const int* idx)
{
  if (w <= 0) return 0;
  idx_table t;
  fill_idx(&t, idx, w);
  unsigned nb = row_blocks(ctx, n, w);
  double* partial = (double*)gb_workspace(ctx, sizeof(double) * (size_t)nb * w);
  if (!partial) return -1;
  dim3 grid(nb, w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  if (dtype == GPU_MV_FLOAT64)
    dot_partial_kernel<double><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n, partial);
  else if (cols_aligned16(X->col, w) && cols_aligned16(Y->col, w))
    dot32_partial_kernel<<<grid, 256, 0, S(ctx)>>>(*X, *Y, n, partial);
  else
    dot_partial_kernel<float><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n, partial);
  dot_reduce_kernel<<<(w + 63) / 64, 64, 0, S(ctx)>>>(partial, nb, t, w, out);
  gb_prof_end(ctx, &pr, (dtype == GPU_MV_FLOAT64 ? 8.0 : 4.0) * n * w * 2, 2.0 * n * w);
  gb_count_launch(2);
  return CUDA_LAUNCH_CHECK(ctx, "dot_cols");
}

// fused residual R = lambda*BX - AX with squared column norms
template <typename T, int OUT32>
struct rr_out {
  typedef T type;
};
template <>
struct rr_out<double, 1> {
  typedef float type;
};

template <typename T, int OUT32 = 0>
__global__ void residual_partial_kernel(blk_cols BX, blk_cols AX, const double* __restrict__ lambda,
                                        idx_table idx, blk_cols R, long n,
                                        double* __restrict__ partial)
{
  // T: arithmetic and input type; the residual is stored as TO (FP32 for the
  // FP64-accumulated explicit phase: its norm is taken before the rounding)
  using TO = typename rr_out<T, OUT32>::type;
  const T* bx = (const T*)BX.col[blockIdx.y];
  const T* ax = (const T*)AX.col[blockIdx.y];
  TO* rr = (TO*)R.col[blockIdx.y];
  const T lam = (T)lambda[idx.v[blockIdx.y]];
  double s = 0.0;
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    T v = lam * bx[r] - ax[r];
    rr[r] = (TO)v;
    s += (double)v * (double)v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

extern "C" int gb_residual(gpu_Context* ctx, int dtype, long n, const blk_cols* BX,
                           const blk_cols* AX, const double* lambda, const int* idx,
                           const blk_cols* R, int w, double* norm2)
{
  if (w <= 0) return 0;
  idx_table t;
  fill_idx(&t, idx, w);
  unsigned nb = row_blocks(ctx, n, w);
  double* partial = (double*)gb_workspace(ctx, sizeof(double) * (size_t)nb * w);
  if (!partial) return -1;
  dim3 grid(nb, w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_RESID);
  if (dtype == GPU_MV_FLOAT64)
    residual_partial_kernel<double><<<grid, 256, 0, S(ctx)>>>(*BX, *AX, lambda, t, *R, n, partial);
  else if (dtype == GPU_MV_FLOAT32)
    residual_partial_kernel<float><<<grid, 256, 0, S(ctx)>>>(*BX, *AX, lambda, t, *R, n, partial);
  else  // FP64 inputs, FP32 residual
    residual_partial_kernel<double, 1><<<grid, 256, 0, S(ctx)>>>(*BX, *AX, lambda, t, *R, n, partial);
  dot_reduce_kernel<<<(w + 63) / 64, 64, 0, S(ctx)>>>(partial, nb, t, w, norm2);
  gb_prof_end(ctx, &pr, (dtype == GPU_MV_FLOAT32 ? 12.0 : (dtype == GPU_MV_FLOAT64 ? 24.0 : 20.0)) * n * w,
              4.0 * n * w);
  gb_count_launch(2);
  return CUDA_LAUNCH_CHECK(ctx, "residual");
}

// Y64 = X64 + D (D FP32), and D <- (float) Y64: the FP64-accumulated block
// update of the explicit phase (the correction carries FP32 rounding
// relative to its own size) and its FP32 shadow
__global__ void acc64_kernel(blk_cols X, blk_cols D, blk_cols Y, long n)
{
  const double* x = (const double*)X.col[blockIdx.y];
  float* d = (float*)D.col[blockIdx.y];
  double* y = (double*)Y.col[blockIdx.y];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    const double v = x[r] + (double)d[r];
    y[r] = v;
    d[r] = (float)v;
  }
}

extern "C" int gb_accumulate64(gpu_Context* ctx, long n, const blk_cols* X64, const blk_cols* D32,
                               const blk_cols* Y64, int w)
{
  if (w <= 0 || n <= 0) return 0;
  dim3 grid(row_blocks(ctx, n, w), w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  acc64_kernel<<<grid, 256, 0, S(ctx)>>>(*X64, *D32, *Y64, n);
  gb_prof_end(ctx, &pr, 24.0 * n * w, (double)n * w);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "accumulate64");
}

// The explicit pencil (G, H) of [X R P] from the exact Gram products of the
// split mode.  Inputs (column-major FP64):
//   Hx = X'[X R P]          (k x m, ld k)
//   Hr = R'[R P AR AP]      (nR x (2 nR + 2 nP), ld nR)
//   Hp = P'[P AP]           (nP x 2 nP, ld nP)
//   Gt(c, i) = S_c' RS_i    (ld ld; column i < k of the tensor-core product
//                            [X R P]'[RS AR AP]), RS = lambda X - A X
// with lambda the Rayleigh quotients of X.  The X rows of G are formed in
// residual form, G(i, c) = X_i' A S_c = lambda_i X_i' S_c - RS_i' S_c, so that
// A X (whose norm is the spectrum's scale) never enters a product and the
// rounding of RS'S scales with the residual (TF32 products suffice there);
// the other blocks are R'AR, R'AP, P'AP.  Symmetric blocks are averaged with
// their transposes.
__global__ void split_pencil_kernel(const double* __restrict__ Hx, const double* __restrict__ Hr,
                                    const double* __restrict__ Hp, const double* __restrict__ Gt,
                                    double* G, double* H, int ld, const double* __restrict__ lam,
                                    int k, int nR, int nP)
{
  const int m = k + nR + nP;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * m) return;
  const int a = e % m, b = e / m;
  double g, h;
  if (a < k || b < k) {
    // Gt = RS' [RS S] (k x (k + m), leading dimension k): S_c' RS_i at
    // Gt[i + (k + c) k]
    if (a < k && b < k) {
      const double h1 = Hx[a + (size_t)b * k], h2 = Hx[b + (size_t)a * k];
      h = 0.5 * (h1 + h2);
      g = 0.5 * ((lam[a] * h1 - Gt[a + (size_t)(k + b) * k]) + (lam[b] * h2 - Gt[b + (size_t)(k + a) * k]));
    } else {
      const int i = a < k ? a : b, c = a < k ? b : a;
      h = Hx[i + (size_t)c * k];
      g = lam[i] * h - Gt[i + (size_t)(k + c) * k];
    }
  } else {
    const int ra = a - k, rb = b - k;  // offsets in [R P]
    if (ra < nR && rb < nR) {
      h = 0.5 * (Hr[ra + (size_t)rb * nR] + Hr[rb + (size_t)ra * nR]);
      const size_t o = (size_t)(nR + nP) * nR;
      g = 0.5 * (Hr[o + ra + (size_t)rb * nR] + Hr[o + rb + (size_t)ra * nR]);
    } else if (ra < nR || rb < nR) {
      const int r = ra < nR ? ra : rb, p = (ra < nR ? rb : ra) - nR;
      h = Hr[r + (size_t)(nR + p) * nR];
      g = Hr[r + (size_t)(2 * nR + nP + p) * nR];
    } else {
      const int pa = ra - nR, pb = rb - nR;
      h = 0.5 * (Hp[pa + (size_t)pb * nP] + Hp[pb + (size_t)pa * nP]);
      g = 0.5 * (Hp[pa + (size_t)(nP + pb) * nP] + Hp[pb + (size_t)(nP + pa) * nP]);
    }
  }
  G[a + (size_t)b * ld] = g;
  H[a + (size_t)b * ld] = h;
}

extern "C" int gb_split_pencil(gpu_Context* ctx, const double* Hx, const double* Hr, const double* Hp,
                               const double* Gt, double* G, double* H, int ld, const double* lam, int k,
                               int nR, int nP)
{
  const int m = k + nR + nP;
  split_pencil_kernel<<<(m * m + 255) / 256, 256, 0, S(ctx)>>>(Hx, Hr, Hp, Gt, G, H, ld, lam, k, nR, nP);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "split pencil");
}

__global__ void rayleigh_kernel(int w, const double* num, const double* den, double* lam)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < w) lam[i] = den[i] > 0.0 ? num[i] / den[i] : 0.0;
}

extern "C" int gb_rayleigh_quotients(gpu_Context* ctx, int dtype, long n, const blk_cols* X,
                                     const blk_cols* AX, int w, double* scratch, double* lam)
{
  int idx[BLK_MAXCOLS];
  for (int c = 0; c < w; c++) idx[c] = c;
  if (gb_dot_cols(ctx, dtype, n, X, AX, w, scratch, idx)) return -1;
  if (gb_dot_cols(ctx, dtype, n, X, X, w, scratch + w, idx)) return -1;
  rayleigh_kernel<<<(w + 127) / 128, 128, 0, S(ctx)>>>(w, scratch, scratch + w, lam);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "rayleigh quotients");
}

template <typename TI, typename TO>
__global__ void convert_kernel(blk_cols X, blk_cols Y, long n)
{
  const TI* x = (const TI*)X.col[blockIdx.y];
  TO* y = (TO*)Y.col[blockIdx.y];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    y[r] = (TO)x[r];
}

extern "C" int gb_convert(gpu_Context* ctx, long n, int dtype_x, const blk_cols* X, int dtype_y,
                          const blk_cols* Y, int w)
{
  if (w <= 0 || n <= 0) return 0;
  dim3 grid(row_blocks(ctx, n, w), w);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_BLAS1);
  if (dtype_x == GPU_MV_FLOAT64 && dtype_y == GPU_MV_FLOAT32)
    convert_kernel<double, float><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n);
  else if (dtype_x == GPU_MV_FLOAT32 && dtype_y == GPU_MV_FLOAT64)
    convert_kernel<float, double><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n);
  else if (dtype_x == GPU_MV_FLOAT64)
    convert_kernel<double, double><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n);
  else
    convert_kernel<float, float><<<grid, 256, 0, S(ctx)>>>(*X, *Y, n);
  gb_prof_end(ctx, &pr, ((dtype_x == GPU_MV_FLOAT64 ? 8.0 : 4.0) + (dtype_y == GPU_MV_FLOAT64 ? 8.0 : 4.0)) * n * w, 0.0);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "convert");
}

// ------------------------------------------------------------------------
// drand48: state_{t+1} = a*state_t + c mod 2^48 with a = 0x5DEECE66D,
// c = 0xB, state_0 = (seed << 16) | 0x330E, value = state / 2^48.
// Element e of the fill (column-major over the listed columns) uses state
// e+1; each thread jumps ahead with the affine-map powers (mod 2^64
// arithmetic is exact mod 2^48).
// ------------------------------------------------------------------------
struct lcg_table {
  unsigned long long a[48], c[48];  // map for 2^b steps
};

__device__ __forceinline__ unsigned long long lcg_jump(const lcg_table& t, unsigned long long s,
                                                       unsigned long long steps)
{
  const unsigned long long M = (1ULL << 48) - 1;
  for (int b = 0; b < 48 && steps; b++, steps >>= 1)
    if (steps & 1) s = (t.a[b] * s + t.c[b]) & M;
  return s;
}

template <typename T>
__global__ void drand48_kernel(T* data, long n, long ld, idx_table idx, int w,
                               unsigned long long state0, lcg_table tab)
{
  const unsigned long long M = (1ULL << 48) - 1;
  const unsigned long long A = 0x5DEECE66DULL, Cc = 0xBULL;
  long total = n * (long)w;
  long per = 64;  // consecutive values per thread
  long first = (blockIdx.x * (long)blockDim.x + threadIdx.x) * per;
  if (first >= total) return;
  unsigned long long s = lcg_jump(tab, state0, (unsigned long long)first);
  long last = min(total, first + per);
  for (long e = first; e < last; e++) {
    s = (A * s + Cc) & M;
    double v = (double)s * (1.0 / 281474976710656.0);
    long c = e / n, r = e - c * n;
    data[(long)idx.v[c] * ld + r] = (T)(2.0 * v - 1.0);
  }
}

extern "C" int gb_drand48_fill(gpu_Context* ctx, int dtype, void* data, long n, long ld,
                               const int* idx, int w, unsigned int seed)
{
  if (w <= 0 || n <= 0) return 0;
  idx_table t;
  fill_idx(&t, idx, w);
  lcg_table tab;
  const unsigned long long M = (1ULL << 48) - 1;
  unsigned long long a = 0x5DEECE66DULL, c = 0xBULL;
  for (int b = 0; b < 48; b++) {
    tab.a[b] = a;
    tab.c[b] = c;
    // compose the map with itself: s -> a(a s + c) + c
    unsigned long long a2 = (a * a) & M, c2 = (a * c + c) & M;
    a = a2;
    c = c2;
  }
  unsigned long long state0 = (((unsigned long long)seed) << 16) | 0x330EULL;
  long total = n * (long)w;
  long threads = (total + 63) / 64;
  unsigned blocks = (unsigned)((threads + 255) / 256);
  if (dtype == GPU_MV_FLOAT64)
    drand48_kernel<double><<<blocks, 256, 0, S(ctx)>>>((double*)data, n, ld, t, w, state0, tab);
  else
    drand48_kernel<float><<<blocks, 256, 0, S(ctx)>>>((float*)data, n, ld, t, w, state0, tab);
  gb_count_launch(1);
  return CUDA_LAUNCH_CHECK(ctx, "drand48_fill");
}

// ------------------------------------------------------------------------
// Gram product that allocates nothing (gpu_GramNoAlloc in lobpcg_gb300.h).
// The split-k partial sums live in this file-scope device array instead of
// the context's cudaMalloc'ed workspace.  Host code must not pass the
// array's name to a kernel (on the host it is only a stand-in symbol); its
// device address is looked up once per device with cudaGetSymbolAddress.
// ------------------------------------------------------------------------
#define GRAM_NOALLOC_SCRATCH_DOUBLES (512 * 1024) /* 4 MiB per device */
static __device__ __align__(256) double g_gram_noalloc_scratch[GRAM_NOALLOC_SCRATCH_DOUBLES];

#define GRAM_NOALLOC_MAX_DEVICES 64
static double* g_noalloc_addr[GRAM_NOALLOC_MAX_DEVICES];

static double* noalloc_scratch(int device)
{
  if (device < 0 || device >= GRAM_NOALLOC_MAX_DEVICES) return NULL;
  if (!g_noalloc_addr[device]) {
    void* p = NULL;
    // the caller's device is current here (cudaGetDevice above)
    if (cudaGetSymbolAddress(&p, g_gram_noalloc_scratch) != cudaSuccess || !p) return NULL;
    g_noalloc_addr[device] = (double*)p;
  }
  return g_noalloc_addr[device];
}

template <typename T, int TM, int TN>
static int gram_noalloc_launch(long n, const blk_cols* X, int h, const blk_cols* Y, int w,
                               double* G, int ldg, double* partial, cudaStream_t stream, int sms)
{
  constexpr int BM = 16 * TM, BN = 16 * TN;
  int gx = (h + BM - 1) / BM, gy = (w + BN - 1) / BN;
  long splits = 2L * sms / (gx * gy);
  long cap = GRAM_NOALLOC_SCRATCH_DOUBLES / ((long)h * w);  // splits that fit the array
  if (splits > cap) splits = cap;
  long max_splits = (n + 255) / 256;
  if (splits > max_splits) splits = max_splits;
  if (splits < 1) splits = 1;
  long rows = (n + splits - 1) / splits;
  rows = (rows + 31) / 32 * 32;
  splits = (n + rows - 1) / rows;
  if (splits < 1) splits = 1;
  dim3 grid(gx, gy, (unsigned)splits);
  // an error left pending by earlier work on this thread is not ours to
  // clear: report it (-3) and leave it for its owner to read
  if (cudaPeekAtLastError() != cudaSuccess) return -3;
  // every partial element of the used splits is written before the
  // reduction reads it, so stale contents from an earlier call never leak
  gram_partial_kernel<T, TM, TN><<<grid, 256, 0, stream>>>(*X, h, *Y, w, n, rows, partial);
  if (cudaGetLastError() != cudaSuccess) return -3;
  gram_reduce_kernel<<<(h * w + 255) / 256, 256, 0, stream>>>(partial, (int)splits, h, w, G, ldg);
  gb_count_launch(2);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

extern "C" int gpu_GramNoAlloc(int dtype, long n, const void* X, long ldx, int h, const void* Y,
                               long ldy, int w, double* G, int ldg, void* stream)
{
  if (n <= 0 || h <= 0 || w <= 0 || !X || !Y || !G || ldx < n || ldy < n || ldg < h ||
      (dtype != GPU_MV_FLOAT64 && dtype != GPU_MV_FLOAT32))
    return -1;
  if (h > BLK_MAXCOLS || w > BLK_MAXCOLS || (long)h * w > GRAM_NOALLOC_SCRATCH_DOUBLES) return -2;
  int device = -1;
  if (cudaGetDevice(&device) != cudaSuccess) return -3;
  double* partial = noalloc_scratch(device);
  if (!partial) return -3;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
    sms = 152;
  const size_t es = dtype == GPU_MV_FLOAT64 ? 8 : 4;
  blk_cols xc, yc;
  for (int c = 0; c < h; c++) xc.col[c] = (const char*)X + es * (size_t)ldx * c;
  for (int c = 0; c < w; c++) yc.col[c] = (const char*)Y + es * (size_t)ldy * c;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == GPU_MV_FLOAT64) {
    if (h <= 32 && w <= 32) return gram_noalloc_launch<double, 2, 2>(n, &xc, h, &yc, w, G, ldg, partial, s, sms);
    return gram_noalloc_launch<double, 4, 4>(n, &xc, h, &yc, w, G, ldg, partial, s, sms);
  }
  if (h <= 32 && w <= 32) return gram_noalloc_launch<float, 2, 2>(n, &xc, h, &yc, w, G, ldg, partial, s, sms);
  return gram_noalloc_launch<float, 4, 4>(n, &xc, h, &yc, w, G, ldg, partial, s, sms);
}
