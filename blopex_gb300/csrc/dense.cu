// dense.cu -- small dense FP64 linear algebra on the device, for the
// (3k x 3k at most) Gram matrices of the solver:
//   * Cholesky-QR factor: upper Cholesky U of a Gram block (A = U'U),
//     then inv(U) with the strict lower part cleared -- the small-matrix
//     half of lobpcg_MultiVectorImplicitQR (lobpcg.c:197-232: dpotrf 'U',
//     utilities_FortranMatrixUpperInv, utilities_FortranMatrixClearL);
//   * generalized symmetric-definite eigensolver A v = w B v (itype 1,
//     lower triangles): Cholesky B = L L', C = inv(L) A inv(L)', cyclic
//     Jacobi on C, eigenvectors inv(L)' V sorted ascending -- replaces the
//     dsygv call of lobpcg_solveGEVP (lobpcg.c:66-103);
//   * symmetrize / identity / diagonal / small GEMM helpers
//     (fortran_matrix.c:313-330, 428-452, 665-685, 1016-1077).
// Each solve runs in one CTA; every loop has a fixed trip count, so no
// kernel here can spin.  Info codes follow LAPACK: the order of the first
// non-positive leading minor, or m + that order for B in the eigensolver,
// or 2m+1 if Jacobi did not converge within its sweep limit.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "internal.h"

static inline cudaStream_t S(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

#define DENSE_THREADS 512

// upper Cholesky of the m x m block at A (ld), reading the upper triangle;
// writes U into the upper triangle.  Returns 0 or the failing order.
__device__ int chol_upper_dev(double* A, int ld, int m)
{
  __shared__ int s_info;
  if (threadIdx.x == 0) s_info = 0;
  __syncthreads();
  for (int j = 0; j < m; j++) {
    // U(j,j) = sqrt(A(j,j) - sum_{p<j} U(p,j)^2)
    if (threadIdx.x == 0) {
      double s = A[j + (size_t)j * ld];
      for (int p = 0; p < j; p++) {
        double u = A[p + (size_t)j * ld];
        s -= u * u;
      }
      if (!(s > 0.0)) {
        s_info = j + 1;
      } else {
        A[j + (size_t)j * ld] = sqrt(s);
      }
    }
    __syncthreads();
    if (s_info) return s_info;
    const double ujj = A[j + (size_t)j * ld];
    // U(j,i) = (A(j,i) - sum_{p<j} U(p,j) U(p,i)) / U(j,j), i > j
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
      double s = A[j + (size_t)i * ld];
      for (int p = 0; p < j; p++) s -= A[p + (size_t)j * ld] * A[p + (size_t)i * ld];
      A[j + (size_t)i * ld] = s / ujj;
    }
    __syncthreads();
  }
  return 0;
}

// lower Cholesky of the m x m block at B (ld), reading the lower triangle.
__device__ int chol_lower_dev(double* B, int ld, int m)
{
  __shared__ int s_info;
  if (threadIdx.x == 0) s_info = 0;
  __syncthreads();
  for (int j = 0; j < m; j++) {
    if (threadIdx.x == 0) {
      double s = B[j + (size_t)j * ld];
      for (int p = 0; p < j; p++) {
        double l = B[j + (size_t)p * ld];
        s -= l * l;
      }
      if (!(s > 0.0))
        s_info = j + 1;
      else
        B[j + (size_t)j * ld] = sqrt(s);
    }
    __syncthreads();
    if (s_info) return s_info;
    const double ljj = B[j + (size_t)j * ld];
    for (int i = j + 1 + threadIdx.x; i < m; i += blockDim.x) {
      double s = B[i + (size_t)j * ld];
      for (int p = 0; p < j; p++) s -= B[i + (size_t)p * ld] * B[j + (size_t)p * ld];
      B[i + (size_t)j * ld] = s / ljj;
    }
    __syncthreads();
  }
  return 0;
}

// A <- inv(U) in place (upper), strict lower cleared.  W: m*m scratch.
__global__ void __launch_bounds__(DENSE_THREADS) cholqr_factor_kernel(double* A, int ld, int m,
                                                                      int* info, double* W,
                                                                      int force_fail)
{
  int rc = chol_upper_dev(A, ld, m);
  if (threadIdx.x == 0) *info = rc ? rc : (force_fail ? 1 : 0);
  if (rc || force_fail) return;
  // column j of inv(U): back substitution, one thread per column
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    double* x = W + (size_t)j * m;
    for (int i = m - 1; i > j; i--) x[i] = 0.0;
    x[j] = 1.0 / A[j + (size_t)j * ld];
    for (int i = j - 1; i >= 0; i--) {
      double s = 0.0;
      for (int l = i + 1; l <= j; l++) s += A[i + (size_t)l * ld] * x[l];
      x[i] = -s / A[i + (size_t)i * ld];
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    int i = e % m, j = e / m;
    A[i + (size_t)j * ld] = (i <= j) ? W[(size_t)j * m + i] : 0.0;
  }
}

// Cholesky of a Gram block that may be (numerically) rank deficient: a
// column whose pivot falls below tol times its diagonal is dropped (its row
// of U is zeroed with a unit diagonal, dropped[j] = 1); then A <- inv(U)
// with the dropped columns zeroed, so that the dropped directions leave the
// basis.  *ndrop = number of dropped columns.
__global__ void __launch_bounds__(DENSE_THREADS) chol_deflate_kernel(double* A, int ld, int m,
                                                                     double tol, int* dropped,
                                                                     int* ndrop, double* W)
{
  __shared__ int s_drop;
  __shared__ int s_cnt;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) s_cnt = 0;
  for (int j = 0; j < m; j++) {
    if (tid == 0) {
      const double d0 = A[j + (size_t)j * ld];
      double s = d0;
      for (int p = 0; p < j; p++) {
        const double u = A[p + (size_t)j * ld];
        s -= u * u;
      }
      s_drop = !(s > tol * d0) || !(d0 > 0.0);
      A[j + (size_t)j * ld] = s_drop ? 1.0 : sqrt(s);
      dropped[j] = s_drop;
      s_cnt += s_drop;
    }
    __syncthreads();
    const int drop = s_drop;
    const double ujj = A[j + (size_t)j * ld];
    for (int i = j + 1 + tid; i < m; i += nt) {
      double v = 0.0;
      if (!drop) {
        v = A[j + (size_t)i * ld];
        for (int p = 0; p < j; p++) v -= A[p + (size_t)j * ld] * A[p + (size_t)i * ld];
        v /= ujj;
      }
      A[j + (size_t)i * ld] = v;
    }
    __syncthreads();
  }
  for (int j = tid; j < m; j += nt) {
    double* x = W + (size_t)j * m;
    for (int i = m - 1; i > j; i--) x[i] = 0.0;
    x[j] = 1.0 / A[j + (size_t)j * ld];
    for (int i = j - 1; i >= 0; i--) {
      double t = 0.0;
      for (int l = i + 1; l <= j; l++) t += A[i + (size_t)l * ld] * x[l];
      x[i] = -t / A[i + (size_t)i * ld];
    }
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    const int i = e % m, j = e / m;
    A[i + (size_t)j * ld] = (i <= j && !dropped[j]) ? W[(size_t)j * m + i] : 0.0;
  }
  if (tid == 0) *ndrop = s_cnt;
}

extern "C" int gb_chol_deflate(gpu_Context* ctx, double* A, int ld, int m, double tol, int* dropped,
                               int* ndrop)
{
  double* W = (double*)gb_workspace(ctx, sizeof(double) * (size_t)m * m + 64);
  if (!W) return -1;
  chol_deflate_kernel<<<1, DENSE_THREADS, 0, S(ctx)>>>(A, ld, m, tol, dropped, ndrop, W);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "chol_deflate");
}

// rows / columns off + j of the pencil (G2, H2) for dropped[j]: decoupled,
// H2_jj = 1 and G2_jj = 2 max_{i<kx} |G2_ii| + 1.  By interlacing with the
// first kx coordinates (H2 = I on them) the kx smallest eigenvalues are at
// most max_{i<kx} G2_ii, so those coordinates take no part in the wanted
// eigenvectors, and the pencil's norm grows by at most a factor ~2.
__global__ void deflate_pencil_kernel(double* G, double* H, int ld, int mtot, int off, int m,
                                      const int* dropped, int kx)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= m * mtot) return;
  const int j = e % m, o = e / m;
  if (!dropped[j]) return;
  double big = 0.0;
  for (int i = 0; i < kx; i++) big = fmax(big, fabs(G[i + (size_t)i * ld]));
  big = 2.0 * big + 1.0;
  const int a = off + j;
  const double g = (o == a) ? big : 0.0, h = (o == a) ? 1.0 : 0.0;
  G[a + (size_t)o * ld] = g;
  G[o + (size_t)a * ld] = g;
  H[a + (size_t)o * ld] = h;
  H[o + (size_t)a * ld] = h;
}

extern "C" int gb_deflate_pencil(gpu_Context* ctx, double* G, double* H, int ld, int mtot, int off,
                                 int m, const int* dropped, int kx)
{
  if (m <= 0) return 0;
  deflate_pencil_kernel<<<(m * mtot + 255) / 256, 256, 0, S(ctx)>>>(G, H, ld, mtot, off, m, dropped, kx);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "deflate_pencil");
}

extern "C" int gb_cholqr_factor(gpu_Context* ctx, double* A, int ld, int m, int* info)
{
  double* W = (double*)gb_workspace(ctx, sizeof(double) * (size_t)m * m + 64);
  if (!W) return -1;
  int force = 0;
  ctx->potrf_calls++;
  if (ctx->opt.potrf_fail_at > 0 && ctx->potrf_calls == ctx->opt.potrf_fail_at) force = 1;
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_CHOLQR);
  cholqr_factor_kernel<<<1, DENSE_THREADS, 0, S(ctx)>>>(A, ld, m, info, W, force);
  gb_prof_end(ctx, &pr, 16.0 * m * m, (double)m * m * m / 1.5);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "cholqr_factor");
}

// ---------------------------------------------------------------------------
// generalized eigensolver
// scratch layout (m x m each, ld m): C (reduced matrix), V (eigenvectors)
// ---------------------------------------------------------------------------
#define JACOBI_MAX_SWEEPS 40

__global__ void __launch_bounds__(DENSE_THREADS) sygv_kernel(double* A, double* B, int ld, int m,
                                                             double* w, int* info, double* C,
                                                             double* V, int force_fail,
                                                             const int* gate, int* count)
{
  // gate: status word of the fast path; this solver runs only when the fast
  // path failed for a reason it can fix (5 = B not positive definite, which
  // the fast path has already reported through *info)
  if (gate && (*gate == 0 || *gate == 5)) return;
  if (gate && threadIdx.x == 0) atomicAdd(&count[2], 1);
  __shared__ double s_c[256], s_s[256];
  __shared__ int s_p[256], s_q[256];
  __shared__ int s_done;
  __shared__ double s_norm;
  __shared__ int s_perm[512];
  const int tid = threadIdx.x, nt = blockDim.x;

  if (force_fail) {
    if (tid == 0) *info = 1;
    return;
  }
  // 1. B = L L' (lower)
  int rc = chol_lower_dev(B, ld, m);
  if (rc) {
    if (tid == 0) *info = m + rc;
    return;
  }
  // 2. C = inv(L) A inv(L)': first X = inv(L) A (A symmetric from its lower
  //    triangle), column by column; then C' = inv(L) X' row by row.
  for (int j = tid; j < m; j += nt) {
    double* x = C + (size_t)j * m;
    for (int i = 0; i < m; i++) {
      double a = (i >= j) ? A[i + (size_t)j * ld] : A[j + (size_t)i * ld];
      for (int p = 0; p < i; p++) a -= B[i + (size_t)p * ld] * x[p];
      x[i] = a / B[i + (size_t)i * ld];
    }
  }
  __syncthreads();
  // V holds X' temporarily: V(:, j) = row j of X
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    V[i + (size_t)j * m] = C[j + (size_t)i * m];
  }
  __syncthreads();
  for (int j = tid; j < m; j += nt) {
    double* x = V + (size_t)j * m;
    double* out = C + (size_t)j * m;
    for (int i = 0; i < m; i++) {
      double a = x[i];
      for (int p = 0; p < i; p++) a -= B[i + (size_t)p * ld] * out[p];
      out[i] = a / B[i + (size_t)i * ld];
    }
  }
  __syncthreads();
  // symmetrize C and set V = I
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    if (i > j) {
      double v = 0.5 * (C[i + (size_t)j * m] + C[j + (size_t)i * m]);
      C[i + (size_t)j * m] = v;
      C[j + (size_t)i * m] = v;
    }
    V[i + (size_t)j * m] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();

  // 3. cyclic Jacobi, round-robin pairing over me = m rounded up to even.
  //    Thresholds are absolute, relative to |C|_F (the backward-error scale
  //    of a LAPACK solve): rotate while |c_pq| > 1e-3 eps |C|_F, converged
  //    once every |c_pq| <= 4 eps |C|_F.
  {
    __shared__ double s_red[DENSE_THREADS];
    double acc = 0.0;
    for (int e = tid; e < m * m; e += nt) acc += C[e] * C[e];
    s_red[tid] = acc;
    __syncthreads();
    for (int o = nt / 2; o > 0; o >>= 1) {
      if (tid < o) s_red[tid] += s_red[tid + o];
      __syncthreads();
    }
    if (tid == 0) s_norm = sqrt(s_red[0]);
    __syncthreads();
  }
  const double thr_rot = 1e-3 * DBL_EPSILON * s_norm;
  const double thr_done = 4.0 * DBL_EPSILON * s_norm;
  const int me = (m + 1) & ~1;
  const int half = me / 2;
  int converged = 0;
  for (int sweep = 0; sweep < JACOBI_MAX_SWEEPS && !converged; sweep++) {
    if (tid == 0) s_done = 1;
    __syncthreads();
    for (int round = 0; round < me - 1; round++) {
      // pair t: positions t and me-1-t of the rotating arrangement; slot 0
      // fixed, the others rotate by `round`
      for (int t = tid; t < half; t += nt) {
        int a = t, b = me - 1 - t;
        int pa = (a == 0) ? 0 : 1 + (a - 1 + round) % (me - 1);
        int pb = (b == 0) ? 0 : 1 + (b - 1 + round) % (me - 1);
        int p = min(pa, pb), q = max(pa, pb);
        double c = 1.0, s = 0.0;
        if (q < m) {
          double apq = C[p + (size_t)q * m];
          double app = C[p + (size_t)p * m], aqq = C[q + (size_t)q * m];
          if (fabs(apq) > thr_rot) {
            double theta = (aqq - app) / (2.0 * apq);
            double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(1.0 + theta * theta));
            c = 1.0 / sqrt(1.0 + tt * tt);
            s = tt * c;
            if (fabs(apq) > thr_done) s_done = 0;
          }
        }
        s_p[t] = p;
        s_q[t] = q;
        s_c[t] = c;
        s_s[t] = s;
      }
      __syncthreads();
      // rows: C <- J' C
      for (int e = tid; e < half * m; e += nt) {
        int t = e / m, j = e % m;
        int p = s_p[t], q = s_q[t];
        double s = s_s[t];
        if (q >= m || s == 0.0) continue;
        double c = s_c[t];
        double ap = C[p + (size_t)j * m], aq = C[q + (size_t)j * m];
        C[p + (size_t)j * m] = c * ap - s * aq;
        C[q + (size_t)j * m] = s * ap + c * aq;
      }
      __syncthreads();
      // columns: C <- C J, V <- V J
      for (int e = tid; e < half * m; e += nt) {
        int t = e / m, i = e % m;
        int p = s_p[t], q = s_q[t];
        double s = s_s[t];
        if (q >= m || s == 0.0) continue;
        double c = s_c[t];
        double ap = C[i + (size_t)p * m], aq = C[i + (size_t)q * m];
        C[i + (size_t)p * m] = c * ap - s * aq;
        C[i + (size_t)q * m] = s * ap + c * aq;
        double vp = V[i + (size_t)p * m], vq = V[i + (size_t)q * m];
        V[i + (size_t)p * m] = c * vp - s * vq;
        V[i + (size_t)q * m] = s * vp + c * vq;
      }
      __syncthreads();
      // the annihilated entries are zero in exact arithmetic
      for (int t = tid; t < half; t += nt) {
        int p = s_p[t], q = s_q[t];
        if (q < m && s_s[t] != 0.0) {
          C[p + (size_t)q * m] = 0.0;
          C[q + (size_t)p * m] = 0.0;
        }
      }
      __syncthreads();
    }
    converged = s_done;
    __syncthreads();
  }
  if (!converged) {
    if (tid == 0) *info = 2 * m + 1;
    return;
  }
  // 4. ascending order: rank of each eigenvalue (ties by index)
  for (int i = tid; i < m; i += nt) {
    double di = C[i + (size_t)i * m];
    int r = 0;
    for (int j = 0; j < m; j++) {
      double dj = C[j + (size_t)j * m];
      if (dj < di || (dj == di && j < i)) r++;
    }
    s_perm[r] = i;
  }
  __syncthreads();
  for (int r = tid; r < m; r += nt) w[r] = C[s_perm[r] + (size_t)s_perm[r] * m];
  // 5. eigenvectors of the pencil: Z = inv(L)' V(:, perm), into A
  for (int r = tid; r < m; r += nt) {
    const double* v = V + (size_t)s_perm[r] * m;
    double* z = A + (size_t)r * ld;
    for (int i = m - 1; i >= 0; i--) {
      double a = v[i];
      for (int p = i + 1; p < m; p++) a -= B[p + (size_t)i * ld] * z[p];
      z[i] = a / B[i + (size_t)i * ld];
    }
  }
  __syncthreads();
  if (tid == 0) *info = 0;
}

/* One-CTA FP64 solver: used for orders the fast path does not take, when
   the fast path's FP32 stage fails (gate != NULL: runs only if *gate != 0),
   and for injected failures (force). */
extern "C" int gb_sygv_fp64(gpu_Context* ctx, double* A, double* B, int ld, int m, double* w,
                            int* info, const int* gate, int force)
{
  if (m > 512) return gb_fail(ctx, "sygv: order %d exceeds 512", m);
  double* scratch = (double*)gb_workspace(ctx, sizeof(double) * (size_t)2 * m * m + 64);
  if (!scratch) return -1;
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, gate ? GB_K_SYGV_FALLBACK : GB_K_SYGV);
  sygv_kernel<<<1, DENSE_THREADS, 0, S(ctx)>>>(A, B, ld, m, w, info, scratch,
                                               scratch + (size_t)m * m, force, gate,
                                               ctx->dcount);
  gb_prof_end(ctx, &pr, 32.0 * m * m, 0.0);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "sygv");
}

// --------------------------------------------------------------- helpers
__global__ void small_symmetrize_kernel(double* A, int ld, int m)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    if (i > j) {
      double v = (A[i + (size_t)j * ld] + A[j + (size_t)i * ld]) * 0.5;
      A[i + (size_t)j * ld] = v;
      A[j + (size_t)i * ld] = v;
    }
  }
}

__global__ void small_identity_kernel(double* A, int ld, int h, int w)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < h * w; e += gridDim.x * blockDim.x) {
    int i = e % h, j = e / h;
    A[i + (size_t)j * ld] = (i == j) ? 1.0 : 0.0;
  }
}

__global__ void small_diag_kernel(double* A, int ld, int m, const double* d)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    A[i + (size_t)j * ld] = (i == j) ? d[i] : 0.0;
  }
}

__global__ void small_gemm_kernel(const double* A, int lda, int ta, const double* B, int ldb,
                                  int tb, double* C, int ldc, int h, int w, int l)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < h * w; e += gridDim.x * blockDim.x) {
    int i = e % h, j = e / h;
    double s = 0.0;
    for (int q = 0; q < l; q++) {
      double a = ta ? A[q + (size_t)i * lda] : A[i + (size_t)q * lda];
      double b = tb ? B[j + (size_t)q * ldb] : B[q + (size_t)j * ldb];
      s += a * b;
    }
    C[i + (size_t)j * ldc] = s;
  }
}

static unsigned small_blocks(int count)
{
  int b = (count + 255) / 256;
  return b < 1 ? 1 : (b > 64 ? 64 : b);
}

extern "C" int gb_small_symmetrize(gpu_Context* ctx, double* A, int ld, int m)
{
  if (m <= 1) return 0;
  small_symmetrize_kernel<<<small_blocks(m * m), 256, 0, S(ctx)>>>(A, ld, m);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "symmetrize");
}

extern "C" int gb_small_identity(gpu_Context* ctx, double* A, int ld, int h, int w)
{
  if (h <= 0 || w <= 0) return 0;
  small_identity_kernel<<<small_blocks(h * w), 256, 0, S(ctx)>>>(A, ld, h, w);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "identity");
}

__global__ void small_add_diag_kernel(double* A, int ld, int m, double alpha)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) A[i + (size_t)i * ld] += alpha;
}

extern "C" int gb_small_add_diag(gpu_Context* ctx, double* A, int ld, int m, double alpha)
{
  if (m <= 0) return 0;
  small_add_diag_kernel<<<(m + 255) / 256, 256, 0, S(ctx)>>>(A, ld, m, alpha);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "add_diag");
}

extern "C" int gb_small_diag(gpu_Context* ctx, double* A, int ld, int m, const double* d)
{
  if (m <= 0) return 0;
  small_diag_kernel<<<small_blocks(m * m), 256, 0, S(ctx)>>>(A, ld, m, d);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "diag");
}

extern "C" int gb_small_gemm(gpu_Context* ctx, const double* A, int lda, int ta, const double* B,
                             int ldb, int tb, double* C, int ldc, int h, int w, int l)
{
  if (h <= 0 || w <= 0) return 0;
  small_gemm_kernel<<<small_blocks(h * w), 256, 0, S(ctx)>>>(A, lda, ta, B, ldb, tb, C, ldc, h, w, l);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "small_gemm");
}

// ---------------------------------------------------------------------------
// explicit-Gram Rayleigh-Ritz helpers (FP32 phase of the mixed mode)
// ---------------------------------------------------------------------------
// d_i = 1/sqrt(H_ii) (1 when H_ii <= 0); Gs = D sym(G) D, Hs = D sym(H) D
__global__ void scale_pencil_kernel(const double* G, const double* H, double* Gs, double* Hs,
                                    double* d, int ld, int m)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    double h = H[i + (size_t)i * ld];
    d[i] = h > 0.0 ? 1.0 / sqrt(h) : 1.0;
  }
  __syncthreads();  // single block launch below
  for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
    int i = e % m, j = e / m;
    double di = d[i], dj = d[j];
    double g = 0.5 * (G[i + (size_t)j * ld] + G[j + (size_t)i * ld]);
    double hh = 0.5 * (H[i + (size_t)j * ld] + H[j + (size_t)i * ld]);
    Gs[i + (size_t)j * ld] = di * g * dj;
    Hs[i + (size_t)j * ld] = (i == j) ? 1.0 : di * hh * dj;
  }
}

extern "C" int gb_scale_pencil(gpu_Context* ctx, const double* G, const double* H, double* Gs,
                               double* Hs, double* d, int ld, int m)
{
  scale_pencil_kernel<<<1, 1024, 0, S(ctx)>>>(G, H, Gs, Hs, d, ld, m);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "scale_pencil");
}

// C(0:m, 0:k) = D C (undo the scaling of the eigenvector coordinates)
__global__ void scale_rows_kernel(double* C, const double* d, int ld, int m, int k)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * k; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    C[i + (size_t)j * ld] *= d[i];
  }
}

extern "C" int gb_scale_rows(gpu_Context* ctx, double* C, const double* d, int ld, int m, int k)
{
  scale_rows_kernel<<<small_blocks(m * k), 256, 0, S(ctx)>>>(C, d, ld, m, k);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "scale_rows");
}

__global__ void small_copy_kernel(const double* A, int lda, double* B, int ldb, int h, int w)
{
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < h * w; e += gridDim.x * blockDim.x) {
    int i = e % h, j = e / h;
    B[i + (size_t)j * ldb] = A[i + (size_t)j * lda];
  }
}

extern "C" int gb_small_copy(gpu_Context* ctx, const double* A, int lda, double* B, int ldb, int h,
                             int w)
{
  if (h <= 0 || w <= 0) return 0;
  small_copy_kernel<<<small_blocks(h * w), 256, 0, S(ctx)>>>(A, lda, B, ldb, h, w);
  gb_count_launch(1);
  return gb_cuda_check(ctx, (int)cudaGetLastError(), "small_copy");
}
