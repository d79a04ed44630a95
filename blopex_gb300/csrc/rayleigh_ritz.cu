// rayleigh_ritz.cu -- the Rayleigh-Ritz eigenproblem A v = w B v (B SPD,
// order m <= 3k) of every LOBPCG iteration, replacing the dsygv call of
// lobpcg_solveGEVP (blopex_abstract/krylov/lobpcg.c:66-103).  Only the
// lowest nev (= k) eigenpairs are used by the caller and computed.
//
// Default solver (rr_method 0), all FP64, the steps of dsygv:
//   1. one CTA: Cholesky B = L L' (its failure is dsygv's INFO m+j)
//   2. multi-CTA triangular solves: C = inv(L) A inv(L)'
//   3. one CTA: Householder reduction C = Q T Q', T tridiagonal
//   4. one warp per eigenvalue: multisection (32 Sturm counts per step)
//      for the nev smallest eigenvalues of T
//   5. one CTA per eigenvalue: inverse iteration on T - lambda I (LU with
//      partial pivoting), then Cholesky-QR (twice) of the nev vectors --
//      the vectors of near-degenerate eigenvalues come from different
//      starts and are orthonormalised together
//   6. one warp per vector: back-transformation by the Householder
//      reflectors, then inv(L)' (dsygv's outputs; B is left intact).
// The FP64 rate of this GPU is 1/64 of its FP32 rate; the one-CTA steps are
// O(m^3) on one SM (about 1.5 ms at m = 192).
//
// rr_method 2, for well-separated spectra: FP32 cyclic Jacobi on C (every
// CTA rotates its own copy and accumulates a slice of the eigenvectors),
// then two rounds of FP64 refinement with S = V'CV and P = V'V,
//   E_ij = (S_ij - l_j P_ij) / (l_j - l_i)   for separated pairs,
//   E_ij = R_ij / 2 with R = I - P           inside clusters,
// clusters diagonalised by FP64 Jacobi (Ogita & Aishima, Japan J. Indust.
// Appl. Math. 2018: each round squares the eigenvector error).  Its FP32
// start carries errors of eps32 |C| / gap, so it fails on pencils whose
// wanted eigenvalues are close compared with |C|.
//
// Whenever a path cannot finish (status word), the one-CTA FP64 Jacobi
// solver of dense.cu runs on the original pencil instead, gated on the
// device status word (no host sync).  Every loop has a fixed trip count.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "internal.h"

static inline cudaStream_t S_(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

#define RR_THREADS 1024
#define RR_MAX_SMEM_M 192  // FP32 Jacobi path (shared-memory copies of C)
#define RR_MAX_M 384       // tridiagonal path
#define JACOBI32_MAX_SWEEPS 30
#define JACOBI64_MAX_SWEEPS 40

// status words (device ints): [0] fast path failed, [1] Jacobi32 sweeps
struct rr_scratch {
  int* count;  // context counters (see internal.h)
  float *C, *V, *lam32;
  double *L64, *LT64, *C64, *W64;
  double *X, *Xn, *TA, *S, *P, *EI, *Q, *F, *J1, *J2, *lam;
  double *d, *e, *tau;  // tridiagonal T and the Householder scalars
  int* status;
};

// ------------------------------------------------------------------ 1.
// FP64 lower Cholesky of B into s.L64 (m x m, ld m); *info = m + j on
// failure (dsygv's convention for a B that is not positive definite).
// The pivot ratio q_j = L_jj^2 / B_jj is the squared sine of the angle
// between basis vector j and the span of the previous ones.  When its
// minimum is below report_below, B is reported as not definite (INFO m+j,
// so that the caller restarts without P); below RR_GRADED_BELOW, C is
// graded beyond what the tridiagonal solver (absolute accuracy
// eps |C|) resolves for the small eigenvalues, and the FP64 Jacobi solver
// (relative accuracy on graded matrices) runs instead (status 7).  Up to
// order RR_CHOL_SMEM_M the factorisation runs in shared memory, then L and
// L' (row-major) are written out.
#define RR_GRADED_BELOW 1e-10
#define RR_CHOL_SMEM_M 160  // the factor in shared memory (m * m doubles) up to this order
template <bool SMEM>
__global__ void __launch_bounds__(RR_THREADS) rr_chol64_kernel(const double* __restrict__ B, int ld,
                                                               int m, rr_scratch s, int* info,
                                                               double report_below)
{
  extern __shared__ double Ls[];
  __shared__ int bad;
  double* L = SMEM ? Ls : s.L64;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double qmin = HUGE_VAL;
  int jmin = 0;
  if (tid == 0) {
    bad = 0;
    s.status[0] = 0;
    atomicAdd(&s.count[3], 1);
  }
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    L[e] = (i >= j) ? B[i + (size_t)j * ld] : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < m; j++) {
    if (tid == 0) {
      double d = L[j + (size_t)j * m];
      if (!(d > 0.0) || !isfinite(d)) {
        bad = j + 1;
      } else {
        L[j + (size_t)j * m] = sqrt(d);
        const double q = d / B[j + (size_t)j * ld];
        if (q < qmin) {
          qmin = q;
          jmin = j;
        }
      }
    }
    __syncthreads();
    if (bad) break;
    const double djj = L[j + (size_t)j * m];
    for (int i = j + 1 + tid; i < m; i += nt) L[i + (size_t)j * m] /= djj;
    __syncthreads();
    // trailing update, a warp per column: L(i, l) -= L(i, j) L(l, j), i >= l > j
    for (int l = j + 1 + warp; l < m; l += nw) {
      const double llj = L[l + (size_t)j * m];
      for (int i = l + lane; i < m; i += 32) L[i + (size_t)l * m] -= L[i + (size_t)j * m] * llj;
    }
    __syncthreads();
  }
  if (tid == 0 && !bad) {
    if (qmin < report_below) {
      bad = jmin + 1;
    } else if (qmin < RR_GRADED_BELOW) {
      s.status[0] = 7;
      atomicAdd(&s.count[4], 1);
    }
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) {
      s.status[0] = 5;
      *info = m + bad;
    }
    return;
  }
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, p = e / m;
    if (SMEM) s.L64[e] = L[e];
    s.LT64[p + (size_t)i * m] = L[e];
  }
}

// triangular solves with the FP64 factor, one warp (one CTA) per right-hand
// side, column-oriented like the reference BLAS dtrsm: once x_i is known it
// is broadcast from its lane and subtracted from the entries still to be
// solved, so no step needs a reduction across the warp.  The right-hand side
// lives in registers (entry p in lane p % 32, slot p / 32; SL = ceil(m / 32)
// slots):
//   mode 0: X = inv(L) Y, Y symmetric read from its lower triangle (ld ldy)
//   mode 1: X = inv(L) Y' (Y m x m, ld ldy)
//   mode 2: X = inv(L)' Y (Y m x m, ld ldy), result to X with leading dim ldx
// The forward sweeps read columns of L (s.L64), the backward sweep columns
// of L' = rows of L (s.LT64, LT[p + i*m] = L(i, p)): contiguous either way.
#define RR_TRSM_SLOTS (RR_MAX_M / 32)
template <int SL>
__global__ void __launch_bounds__(32) rr_trsm64_kernel(int mode, const double* __restrict__ Y,
                                                       int ldy, double* __restrict__ X, int ldx,
                                                       int m, int ncols, rr_scratch s)
{
  if (s.status[0]) return;
  const int lane = threadIdx.x;
  const int j = blockIdx.x;
  if (j >= ncols) return;
  double y[SL];
#pragma unroll
  for (int q = 0; q < SL; q++) {
    const int p = q * 32 + lane;
    double a = 0.0;
    if (p < m) {
      if (mode == 0)
        a = (p >= j) ? Y[p + (size_t)j * ldy] : Y[j + (size_t)p * ldy];
      else if (mode == 1)
        a = Y[j + (size_t)p * ldy];
      else
        a = Y[p + (size_t)j * ldy];
    }
    y[q] = a;
  }
  if (mode < 2) {
    const double* L = s.L64;
#pragma unroll
    for (int q = 0; q < SL; q++) {
      for (int il = 0; il < 32; il++) {
        const int i = q * 32 + il;
        if (i >= m) break;
        const double* li = L + (size_t)i * m;
        const double xi = __shfl_sync(0xffffffffu, y[q], il) / li[i];
        if (lane == il) y[q] = xi;
#pragma unroll
        for (int q2 = q; q2 < SL; q2++) {
          const int p = q2 * 32 + lane;
          if (p > i && p < m) y[q2] -= li[p] * xi;
        }
      }
    }
  } else {
    const double* LT = s.LT64;
#pragma unroll
    for (int q = SL - 1; q >= 0; q--) {
      for (int il = 31; il >= 0; il--) {
        const int i = q * 32 + il;
        if (i >= m) continue;
        const double* lti = LT + (size_t)i * m;  // lti[p] = L(i, p)
        const double xi = __shfl_sync(0xffffffffu, y[q], il) / lti[i];
        if (lane == il) y[q] = xi;
#pragma unroll
        for (int q2 = 0; q2 <= q; q2++) {
          const int p = q2 * 32 + lane;
          if (p < i) y[q2] -= lti[p] * xi;
        }
      }
    }
  }
  double* x = X + (size_t)j * ldx;
#pragma unroll
  for (int q = 0; q < SL; q++) {
    const int p = q * 32 + lane;
    if (p < m) x[p] = y[q];
  }
}

// symmetrise the FP64 reduced matrix and make the FP32 copy for Jacobi
__global__ void rr_sym_kernel(int m, rr_scratch s)
{
  if (s.status[0]) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    double v = 0.5 * (s.C64[i + (size_t)j * m] + s.C64[j + (size_t)i * m]);
    s.C[e] = (float)v;
  }
}

__global__ void rr_sym_store_kernel(int m, rr_scratch s)
{
  if (s.status[0]) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    if (i > j) {
      double v = 0.5 * (s.C64[i + (size_t)j * m] + s.C64[j + (size_t)i * m]);
      s.C64[i + (size_t)j * m] = v;
      s.C64[j + (size_t)i * m] = v;
    }
  }
}

// ------------------------------------------------------------------ 2.
// one Jacobi round schedule: pair t of round r over me (even) slots
__device__ __forceinline__ void rr_pair(int t, int round, int me, int* p, int* q)
{
  int a = t, b = me - 1 - t;
  int pa = (a == 0) ? 0 : 1 + (a - 1 + round) % (me - 1);
  int pb = (b == 0) ? 0 : 1 + (b - 1 + round) % (me - 1);
  *p = min(pa, pb);
  *q = max(pa, pb);
}


// One cyclic-Jacobi sweep structure shared by the FP32 and FP64 solvers.
// A round pairs every index with one partner (tournament ordering); the
// rotations of a round are disjoint, so C <- J' C J is applied as
// independent 2x2 blocks (rows of pair t, columns of pair u): one pass and
// two barriers per round.  Columns of V (rows r0..r0+nr of it) rotate in
// the same pass.  C is m x m with leading dimension lc; V rows have stride lv.
template <typename T>
__device__ int rr_jacobi_rounds(T* C, int m, int lc, T* V, int nr, int lv, T thr_rot,
                                T thr_done, int max_sweeps, T* s_c, T* s_s, int* s_p, int* s_q,
                                int* s_done, int* sweeps_out)
{
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarp = nt >> 5;
  const int me = (m + 1) & ~1, half = me / 2;
  int converged = 0, sweep = 0;
  for (; sweep < max_sweeps && !converged; sweep++) {
    if (tid == 0) *s_done = 1;
    __syncthreads();
    for (int round = 0; round < me - 1; round++) {
      for (int t = tid; t < half; t += nt) {
        int p, q;
        rr_pair(t, round, me, &p, &q);
        T c = T(1), sn = T(0);
        if (q < m) {
          T apq = C[p + q * lc], app = C[p + p * lc], aqq = C[q + q * lc];
          if (fabs((double)apq) > (double)thr_rot) {
            T theta = (aqq - app) / (T(2) * apq);
            T tt = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(T(1) + theta * theta));
            c = T(1) / sqrt(T(1) + tt * tt);
            sn = tt * c;
            if (fabs((double)apq) > (double)thr_done) *s_done = 0;
          }
        } else {
          q = p;  // the dummy partner of an odd order
        }
        s_p[t] = p;
        s_q[t] = q;
        s_c[t] = c;
        s_s[t] = sn;
      }
      __syncthreads();
      // 2x2 blocks (pair t rows, pair u columns): warp strides t, lane strides u
      for (int t = warp; t < half; t += nwarp) {
        const int p = s_p[t], q = s_q[t];
        const T ct = s_c[t], st = s_s[t];
        for (int u = lane; u < half; u += 32) {
          const T su = s_s[u];
          if (st == T(0) && su == T(0)) continue;
          const int pu = s_p[u], qu = s_q[u];
          const T cu = s_c[u];
          const int twoq = (q != p), twou = (qu != pu);
          T a = C[p + pu * lc], b = twou ? C[p + qu * lc] : T(0);
          T c2 = twoq ? C[q + pu * lc] : T(0), d = (twoq && twou) ? C[q + qu * lc] : T(0);
          // right rotation by pair u (columns pu, qu)
          T a1 = cu * a - su * b, b1 = su * a + cu * b;
          T c1 = cu * c2 - su * d, d1 = su * c2 + cu * d;
          // left rotation by pair t (rows p, q)
          T a2 = ct * a1 - st * c1, c3 = st * a1 + ct * c1;
          T b2 = ct * b1 - st * d1, d2 = st * b1 + ct * d1;
          if (t == u && twoq) {  // the annihilated entry
            b2 = T(0);
            c3 = T(0);
          }
          C[p + pu * lc] = a2;
          if (twou) C[p + qu * lc] = b2;
          if (twoq) C[q + pu * lc] = c3;
          if (twoq && twou) C[q + qu * lc] = d2;
        }
      }
      // V <- V J for the local rows: warp strides rows, lane strides pairs
      for (int r = warp; r < nr; r += nwarp) {
        for (int u = lane; u < half; u += 32) {
          const T su = s_s[u];
          if (su == T(0)) continue;
          const int pu = s_p[u], qu = s_q[u];
          const T cu = s_c[u];
          T vp = V[r * lv + pu], vq = V[r * lv + qu];
          V[r * lv + pu] = cu * vp - su * vq;
          V[r * lv + qu] = su * vp + cu * vq;
        }
      }
      __syncthreads();
    }
    converged = *s_done;
    __syncthreads();
  }
  *sweeps_out = sweep;
  return converged;
}

// shared-memory layouts use an odd leading dimension so that both the row
// and the column sweeps of a rotation hit 32 different banks
__host__ __device__ __forceinline__ int rr_pad(int m) { return m | 1; }

__global__ void __launch_bounds__(RR_THREADS) rr_jacobi32_kernel(int m, int rows, rr_scratch s)
{
  extern __shared__ float sm[];
  const int lc = rr_pad(m);
  float* Cs = sm;             // m x m, column-major, leading dimension lc
  float* Vs = sm + m * lc;    // rows x m slice of V, row r at Vs + r*lc (V^T layout)
  __shared__ float s_c[256], s_s[256];
  __shared__ int s_p[256], s_q[256];
  __shared__ int s_done;
  __shared__ float s_red[RR_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int r0 = blockIdx.x * rows;
  const int nr = min(rows, m - r0);
  if (s.status[0]) return;
  for (int j = 0; j < m; j++)
    for (int i = tid; i < m; i += nt) Cs[i + j * lc] = s.C[i + (size_t)j * m];
  for (int r = 0; r < rows; r++)
    for (int c = tid; c < m; c += nt) Vs[r * lc + c] = (r0 + r == c) ? 1.f : 0.f;
  float acc = 0.f;
  for (int e = tid; e < m * m; e += nt) acc += s.C[e] * s.C[e];
  s_red[tid] = acc;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) s_red[tid] += s_red[tid + o];
    __syncthreads();
  }
  const float nrm = sqrtf(s_red[0]);
  int sweeps = 0;
  int converged = rr_jacobi_rounds<float>(Cs, m, lc, Vs, nr, lc, 0.05f * FLT_EPSILON * nrm,
                                          8.f * FLT_EPSILON * nrm, JACOBI32_MAX_SWEEPS, s_c, s_s,
                                          s_p, s_q, &s_done, &sweeps);
  if (!converged) {
    if (tid == 0) s.status[0] = 2;
    return;
  }
  for (int r = 0; r < nr; r++)
    for (int c = tid; c < m; c += nt) s.V[(r0 + r) + (size_t)c * m] = Vs[r * lc + c];
  if (blockIdx.x == 0) {
    for (int i = tid; i < m; i += nt) s.lam32[i] = Cs[i + i * lc];
    if (tid == 0) {
      s.status[1] = sweeps;
      atomicAdd(&s.count[0], sweeps);
    }
  }
}

// ------------------------------------------------------------------ 3.
// eigenvectors of C sorted by the FP32 eigenvalues, widened to FP64
__global__ void __launch_bounds__(RR_THREADS) rr_vsort_kernel(int m, rr_scratch s)
{
  __shared__ int perm[512];
  const int tid = threadIdx.x, nt = blockDim.x;
  if (s.status[0]) return;
  for (int i = tid; i < m; i += nt) {
    float di = s.lam32[i];
    int r = 0;
    for (int j = 0; j < m; j++) {
      float dj = s.lam32[j];
      if (dj < di || (dj == di && j < i)) r++;
    }
    perm[r] = i;
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, r = e / m;
    s.X[i + (size_t)r * m] = (double)s.V[i + (size_t)perm[r] * m];
  }
}

// ------------------------------------------------------------------ 4.
// FP64 C(MxN) = op(A) B: amode 0 = A (M x K, lda), 1 = A' with A stored
// K x M (lda), 2 = A symmetric M x M read from its lower triangle.
struct rr_gemm_t {
  const double* A;
  int lda, amode;
  const double* B;
  int ldb;
  double* C;
  int ldc;
  int M, N, K;
};

__global__ void __launch_bounds__(256) rr_gemm_kernel(rr_gemm_t g0, rr_gemm_t g1, const int* status)
{
  if (status[0]) return;
  const rr_gemm_t g = blockIdx.z == 0 ? g0 : g1;
  __shared__ double As[32][33], Bs[32][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
  if (i0 >= g.M || j0 >= g.N) return;
  double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int k0 = 0; k0 < g.K; k0 += 32) {
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      int ii = e % 32, kk = e / 32;
      int i = i0 + ii, k = k0 + kk;
      double v = 0.0;
      if (i < g.M && k < g.K) {
        if (g.amode == 0)
          v = g.A[i + (size_t)k * g.lda];
        else if (g.amode == 1)
          v = g.A[k + (size_t)i * g.lda];
        else
          v = (i >= k) ? g.A[i + (size_t)k * g.lda] : g.A[k + (size_t)i * g.lda];
      }
      As[ii][kk] = v;
      int jj = e / 32, kb = e % 32;
      int j = j0 + jj, k2 = k0 + kb;
      Bs[kb][jj] = (j < g.N && k2 < g.K) ? g.B[k2 + (size_t)j * g.ldb] : 0.0;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; kk++) {
      double a0 = As[ty][kk], a1 = As[ty + 16][kk];
      double b0 = Bs[kk][tx], b1 = Bs[kk][tx + 16];
      acc[0][0] = fma(a0, b0, acc[0][0]);
      acc[0][1] = fma(a0, b1, acc[0][1]);
      acc[1][0] = fma(a1, b0, acc[1][0]);
      acc[1][1] = fma(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
  for (int a = 0; a < 2; a++)
    for (int b = 0; b < 2; b++) {
      int i = i0 + ty + 16 * a, j = j0 + tx + 16 * b;
      if (i < g.M && j < g.N) g.C[i + (size_t)j * g.ldc] = acc[a][b];
    }
}

// FP64 cyclic Jacobi on the c x c matrix M (leading dimension lm); V (same
// layout) receives the eigenvectors as columns.  All threads of the block.
__device__ int rr_jacobi64(double* M, double* V, int c, int lm)
{
  __shared__ double j_c[256], j_s[256];
  __shared__ int j_p[256], j_q[256];
  __shared__ int j_done;
  __shared__ double j_red[RR_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  // V^T is accumulated (row r of V^T = column r of V) so that the generic
  // rounds rotate its columns; transposed back at the end
  for (int e = tid; e < c * c; e += nt) V[(e % c) + (e / c) * lm] = (e % c == e / c) ? 1.0 : 0.0;
  double acc = 0.0;
  for (int e = tid; e < c * c; e += nt) {
    double v = M[(e % c) + (e / c) * lm];
    acc += v * v;
  }
  j_red[tid] = acc;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) j_red[tid] += j_red[tid + o];
    __syncthreads();
  }
  const double nrm = sqrt(j_red[0]);
  int sweeps = 0;
  int ok = rr_jacobi_rounds<double>(M, c, lm, V, c, lm, 1e-3 * DBL_EPSILON * nrm,
                                    4.0 * DBL_EPSILON * nrm, JACOBI64_MAX_SWEEPS, j_c, j_s, j_p,
                                    j_q, &j_done, &sweeps);
  // V holds V^T row-wise: V[r*lm + j] = (V^T)_{r j} = V_{j r}; make it V_{i r} at [i + r*lm]
  for (int e = tid; e < c * c; e += nt) {
    int i = e % c, r = e / c;
    if (i < r) {
      double a = V[i + r * lm], b = V[r + i * lm];
      V[i + r * lm] = b;
      V[r + i * lm] = a;
    }
  }
  __syncthreads();
  return ok;
}

// refinement step: S = X'AX, P = X'BX -> EI = I + E, Q (block diagonal on
// the clusters), lam
#define RR_CLUSTER_SMEM 96

__global__ void __launch_bounds__(RR_THREADS) rr_refine_kernel(int m, rr_scratch s, int last)
{
  extern __shared__ double csm[];  // 2 x RR_CLUSTER_SMEM x rr_pad(RR_CLUSTER_SMEM)
  __shared__ double lt[512];
  __shared__ int cstart[513];
  __shared__ int ncl;
  __shared__ double s_red[RR_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  if (s.status[0]) return;
  const double* S = s.S;
  const double* P = s.P;
  for (int i = tid; i < m; i += nt) lt[i] = S[i + (size_t)i * m] / P[i + (size_t)i * m];
  __syncthreads();
  double mx = 0.0;
  for (int i = tid; i < m; i += nt) mx = fmax(mx, fabs(lt[i]));
  s_red[tid] = mx;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) s_red[tid] = fmax(s_red[tid], s_red[tid + o]);
    __syncthreads();
  }
  // close values are refined together: the first-order correction of a pair
  // is (FP32 error ~1e-7 |C|) / gap, kept below ~1e-2
  const double delta = 2e-5 * s_red[0] + 1e-300;
  if (tid == 0) {
    int n = 0;
    cstart[n++] = 0;
    for (int i = 1; i < m; i++)
      if (lt[i] - lt[i - 1] > delta) cstart[n++] = i;
    cstart[n] = m;
    ncl = n;
  }
  __syncthreads();
  // cluster id of every index
  __shared__ short cid[512];
  for (int c = tid; c < ncl; c += nt)
    for (int i = cstart[c]; i < cstart[c + 1]; i++) cid[i] = (short)c;
  __syncthreads();
  double emax = 0.0;
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    double v;
    if (i == j)
      v = 1.0 + 0.5 * (1.0 - P[e]);
    else if (cid[i] == cid[j])
      v = -0.5 * P[e];
    else
      v = (S[e] - lt[j] * P[e]) / (lt[j] - lt[i]);
    if (i != j) emax = fmax(emax, fabs(v));
    s.EI[e] = v;
    s.Q[e] = (i == j) ? 1.0 : 0.0;
  }
  // the last round must only polish: a correction this large means the
  // FP32 start was too poor (ill-conditioned B); the FP64 solver takes over
  __syncthreads();
  s_red[tid] = emax;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) s_red[tid] = fmax(s_red[tid], s_red[tid + o]);
    __syncthreads();
  }
  if (last && !(s_red[0] <= 1e-8)) {
    if (tid == 0) s.status[0] = 4;
    return;
  }
  for (int i = tid; i < m; i += nt) s.lam[i] = lt[i];
  __syncthreads();
  // clusters: diagonalise S_cc + (R_cc S_cc + S_cc R_cc)/2, R = I - P
  for (int c = 0; c < ncl; c++) {
    const int a0 = cstart[c], sz = cstart[c + 1] - a0;
    if (sz < 2) continue;
    if (tid == 0) atomicMax(&s.count[1], sz);
    const int small = sz <= RR_CLUSTER_SMEM;
    const int lm = small ? rr_pad(sz) : sz;
    double* Mc = small ? csm : s.J1;
    double* Vc = small ? csm + RR_CLUSTER_SMEM * rr_pad(RR_CLUSTER_SMEM) : s.J2;
    // M_c = S + (R S + S R)/2 with R = I - P:  M_c = 2S - (P S + (P S)')/2,
    // S, P symmetric; P S staged through the eigenvector buffer
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      Mc[a + b * lm] = S[(a0 + a) + (size_t)(a0 + b) * m];
      Vc[a + b * lm] = P[(a0 + a) + (size_t)(a0 + b) * m];
    }
    __syncthreads();
    double* PS = s.F;  // sz x sz, leading dimension sz (F is written only later)
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      double t = 0.0;
      for (int l = 0; l < sz; l++) t += Vc[a + l * lm] * Mc[l + b * lm];
      PS[a + b * sz] = t;
    }
    __syncthreads();
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      Mc[a + b * lm] = 2.0 * Mc[a + b * lm] - 0.5 * (PS[a + b * sz] + PS[b + a * sz]);
    }
    __syncthreads();
    // symmetrise
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      if (a > b) {
        double v = 0.5 * (Mc[a + b * lm] + Mc[b + a * lm]);
        Mc[a + b * lm] = v;
        Mc[b + a * lm] = v;
      }
    }
    __syncthreads();
    int ok = rr_jacobi64(Mc, Vc, sz, lm);
    if (!ok) {
      if (tid == 0) s.status[0] = 3;
      return;
    }
    // ascending order inside the cluster
    __shared__ int cperm[512];
    for (int a = tid; a < sz; a += nt) {
      double da = Mc[a + a * lm];
      int r = 0;
      for (int b = 0; b < sz; b++) {
        double db = Mc[b + b * lm];
        if (db < da || (db == da && b < a)) r++;
      }
      cperm[r] = a;
    }
    __syncthreads();
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, r = e / sz;
      s.Q[(a0 + a) + (size_t)(a0 + r) * m] = Vc[a + cperm[r] * lm];
    }
    for (int r = tid; r < sz; r += nt) s.lam[a0 + r] = Mc[cperm[r] + cperm[r] * lm];
    __syncthreads();
  }
}

__global__ void rr_finish_kernel(int nev, rr_scratch s, double* w, int* info)
{
  if (s.status[0]) return;  // the FP64 fallback writes the outputs
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nev; i += gridDim.x * blockDim.x)
    w[i] = s.lam[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) *info = 0;
}

// ------------------------------------------------------ tridiagonal path
__device__ __forceinline__ double rr_warp_sum(double v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum (all threads return it); red holds one double per warp
__device__ double rr_block_sum(double v, double* red)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = rr_warp_sum(v);
  __syncthreads();  // red may still be read by a previous call
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; w++) t += red[w];
  return t;
}

// 3. Householder reduction of the symmetric C (s.C64, lower triangle used,
// ld m) to tridiagonal form, one CTA.  Step j reflects rows/columns j+1..m-1
// with H_j = I - tau_j v v', v = (1, C[j+2.., j] / (alpha - beta)); v is
// stored below the subdiagonal of column j.  Per step: p = tau A22 v in
// two coalesced passes over the lower triangle (column sums, then row sums
// of the strict part), w = p - (tau/2)(p'v) v, A22 -= v w' + w v'.
#define RR_TRD_THREADS 512
__global__ void __launch_bounds__(RR_TRD_THREADS) rr_tridiag_kernel(int m, rr_scratch s)
{
  __shared__ double v[RR_MAX_M], p[RR_MAX_M];
  __shared__ double red[RR_TRD_THREADS / 32];
  __shared__ double sh_tau, sh_scale;
  if (s.status[0]) return;
  double* A = s.C64;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nw = nt >> 5;
  for (int j = 0; j + 2 < m; j++) {
    const int n1 = m - j - 1;
    double* col = A + (size_t)j * m + (j + 1);  // x = col[0 .. n1)
    double acc = 0.0;
    for (int i = 1 + tid; i < n1; i += nt) acc += col[i] * col[i];
    acc = rr_block_sum(acc, red);
    if (tid == 0) {
      const double alpha = col[0];
      double tau = 0.0, beta = alpha, scale = 0.0;
      if (acc > 0.0) {
        beta = -copysign(hypot(alpha, sqrt(acc)), alpha);
        tau = (beta - alpha) / beta;
        scale = 1.0 / (alpha - beta);
      }
      s.d[j] = A[j + (size_t)j * m];
      s.e[j] = beta;
      s.tau[j] = tau;
      sh_tau = tau;
      sh_scale = scale;
    }
    __syncthreads();
    const double tau = sh_tau, scale = sh_scale;
    if (tau == 0.0) continue;  // uniform: x is already reduced
    for (int i = tid; i < n1; i += nt) {
      const double vi = (i == 0) ? 1.0 : col[i] * scale;
      v[i] = vi;
      if (i > 0) col[i] = vi;
    }
    __syncthreads();
    double* A22 = A + (size_t)(j + 1) * m + (j + 1);  // (r, c) at A22[r + c*m]
    // column part: p[c] = sum_{r >= c} A22(r, c) v[r]
    for (int c = warp; c < n1; c += nw) {
      const double* ac = A22 + (size_t)c * m;
      double t = 0.0;
      for (int r = c + lane; r < n1; r += 32) t += ac[r] * v[r];
      t = rr_warp_sum(t);
      if (lane == 0) p[c] = t;
    }
    __syncthreads();
    // row part: + sum_{c < r} A22(r, c) v[c]; then p = tau * p
    for (int r = tid; r < n1; r += nt) {
      double t = 0.0;
      for (int c = 0; c < r; c++) t += A22[r + (size_t)c * m] * v[c];
      p[r] = tau * (p[r] + t);
    }
    __syncthreads();
    acc = 0.0;
    for (int i = tid; i < n1; i += nt) acc += p[i] * v[i];
    const double K = 0.5 * tau * rr_block_sum(acc, red);
    for (int i = tid; i < n1; i += nt) p[i] -= K * v[i];  // p <- w
    __syncthreads();
    for (int c = warp; c < n1; c += nw) {
      double* ac = A22 + (size_t)c * m;
      const double vc = v[c], wc = p[c];
      for (int r = c + lane; r < n1; r += 32) ac[r] -= v[r] * wc + p[r] * vc;
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (m >= 2) {
      s.d[m - 2] = A[(m - 2) + (size_t)(m - 2) * m];
      s.e[m - 2] = A[(m - 1) + (size_t)(m - 2) * m];
      s.tau[m - 2] = 0.0;
    }
    s.d[m - 1] = A[(m - 1) + (size_t)(m - 1) * m];
  }
}

// The same reduction with the lower triangle packed in shared memory
// (column c starts at c*m - c(c-1)/2), for m <= RR_TRD_SMEM_M.  On this GPU a
// warp-wide FP64 instruction occupies the FP64 pipe ~16 cycles whatever its
// lane count, so the passes avoid shuffle-tree reductions: p = A22 v is one
// thread per row (column part j <= i reads consecutive addresses across the
// warp, row part j > i walks the thread's own column), the two scalar sums
// are done by warp 0 alone.
#define RR_TRD_SMEM_M 224
__device__ __forceinline__ int rr_pk(int r, int c, int m) { return c * m - ((c * (c - 1)) >> 1) + (r - c); }

// sum over threads of v, computed by warp 0 from per-thread values staged in
// buf (blockDim.x entries); all threads return the sum
__device__ double rr_sum_w0(double v, double* buf, double* out)
{
  const int tid = threadIdx.x;
  buf[tid] = v;
  __syncthreads();
  if (tid < 32) {
    double t = 0.0;
    for (int i = tid; i < (int)blockDim.x; i += 32) t += buf[i];
    t = rr_warp_sum(t);
    if (tid == 0) *out = t;
  }
  __syncthreads();
  return *out;
}

__global__ void __launch_bounds__(RR_TRD_THREADS) rr_tridiag_smem_kernel(int m, rr_scratch s)
{
  extern __shared__ double Lp[];  // packed lower triangle, m(m+1)/2
  __shared__ double v[RR_TRD_SMEM_M], p[RR_TRD_SMEM_M];
  __shared__ double buf[RR_TRD_THREADS];
  __shared__ double sh_sum, sh_tau, sh_scale;
  if (s.status[0]) return;
  double* A = s.C64;
  const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nw = nt >> 5;
  for (int c = warp; c < m; c += nw)
    for (int r = c + lane; r < m; r += 32) Lp[rr_pk(r, c, m)] = A[r + (size_t)c * m];
  __syncthreads();
  for (int j = 0; j + 2 < m; j++) {
    const int n1 = m - j - 1, o = j + 1;  // trailing block rows/cols o .. m-1
    const int cj = rr_pk(o, j, m);        // x = Lp[cj .. cj + n1)
    if (warp == 0) {
      double acc = 0.0;
      for (int i = 1 + lane; i < n1; i += 32) acc += Lp[cj + i] * Lp[cj + i];
      acc = rr_warp_sum(acc);
      if (lane == 0) {
        const double alpha = Lp[cj];
        double tau = 0.0, beta = alpha, scale = 0.0;
        if (acc > 0.0) {
          beta = -copysign(hypot(alpha, sqrt(acc)), alpha);
          tau = (beta - alpha) / beta;
          scale = 1.0 / (alpha - beta);
        }
        s.d[j] = Lp[rr_pk(j, j, m)];
        s.e[j] = beta;
        s.tau[j] = tau;
        sh_tau = tau;
        sh_scale = scale;
      }
    }
    __syncthreads();
    const double tau = sh_tau, scale = sh_scale;
    if (tau == 0.0) continue;  // uniform
    for (int i = tid; i < n1; i += nt) {
      const double vi = (i == 0) ? 1.0 : Lp[cj + i] * scale;
      v[i] = vi;
      if (i > 0) A[(o + i) + (size_t)j * m] = vi;  // reflector for the back-transformation
    }
    __syncthreads();
    // p_i = tau * (sum_{c <= i} A22(i, c) v_c + sum_{r > i} A22(r, i) v_r)
    double pv = 0.0;
    for (int i = tid; i < n1; i += nt) {
      double t = 0.0;
      int a = rr_pk(o + i, o, m);  // (i, c = 0)
      for (int c = 0; c <= i; c++) {
        t += Lp[a] * v[c];
        a += m - (o + c) - 1;  // next column, same row
      }
      const int b = rr_pk(o + i, o + i, m);
      for (int r = i + 1; r < n1; r++) t += Lp[b + (r - i)] * v[r];
      t *= tau;
      p[i] = t;
      pv += t * v[i];
    }
    const double K = 0.5 * tau * rr_sum_w0(pv, buf, &sh_sum);  // (its barriers order p)
    for (int i = tid; i < n1; i += nt) p[i] -= K * v[i];     // p <- w
    __syncthreads();
    // A22 -= v w' + w v' (lower): warp per column
    for (int c = warp; c < n1; c += nw) {
      const int base = rr_pk(o + c, o + c, m) - c;
      const double vc = v[c], wc = p[c];
      for (int r = c + lane; r < n1; r += 32) Lp[base + r] -= v[r] * wc + p[r] * vc;
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (m >= 2) {
      s.d[m - 2] = Lp[rr_pk(m - 2, m - 2, m)];
      s.e[m - 2] = Lp[rr_pk(m - 1, m - 2, m)];
      s.tau[m - 2] = 0.0;
    }
    s.d[m - 1] = Lp[rr_pk(m - 1, m - 1, m)];
  }
}

// number of eigenvalues of T below x (Sturm count of the LDL' pivots)
__device__ __forceinline__ int rr_sturm(const double* d, const double* e2, int m, double x,
                                        double pivmin)
{
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  int cnt = q < 0.0;
  for (int i = 1; i < m; i++) {
    q = (d[i] - x) - e2[i - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    cnt += q < 0.0;
  }
  return cnt;
}

// 4. eigenvalue j of T (ascending) by multisection: the 32 lanes count at
// 31 interior points of [lo, hi]; the bracket shrinks 32-fold per step
__global__ void __launch_bounds__(32) rr_bisect_kernel(int m, rr_scratch s)
{
  __shared__ double d[RR_MAX_M], e2[RR_MAX_M];
  if (s.status[0]) return;
  const int lane = threadIdx.x, j = blockIdx.x;
  double emax2 = 0.0, glo = HUGE_VAL, ghi = -HUGE_VAL;
  for (int i = lane; i < m; i += 32) {
    const double di = s.d[i];
    const double el = i > 0 ? fabs(s.e[i - 1]) : 0.0, er = i + 1 < m ? fabs(s.e[i]) : 0.0;
    d[i] = di;
    if (i + 1 < m) {
      e2[i] = s.e[i] * s.e[i];
      emax2 = fmax(emax2, e2[i]);
    }
    glo = fmin(glo, di - el - er);
    ghi = fmax(ghi, di + el + er);
  }
  for (int o = 16; o > 0; o >>= 1) {
    emax2 = fmax(emax2, __shfl_xor_sync(0xffffffffu, emax2, o));
    glo = fmin(glo, __shfl_xor_sync(0xffffffffu, glo, o));
    ghi = fmax(ghi, __shfl_xor_sync(0xffffffffu, ghi, o));
  }
  __syncwarp();
  const double pivmin = DBL_MIN * fmax(1.0, emax2);
  const double tnorm = fmax(fabs(glo), fabs(ghi));
  const double pad = 2.0 * DBL_EPSILON * tnorm * m + 2.0 * pivmin;
  double lo = glo - pad, hi = ghi + pad;
  for (int step = 0; step < 16; step++) {
    if (hi - lo <= fmax(2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)), 0.25 * DBL_EPSILON * tnorm))
      break;
    const double x = (lane == 31) ? hi : lo + (hi - lo) * (double)(lane + 1) * (1.0 / 32.0);
    const int cnt = (lane == 31) ? m : rr_sturm(d, e2, m, x, pivmin);
    const unsigned ge = __ballot_sync(0xffffffffu, cnt >= j + 1);
    const int f = __ffs(ge) - 1;  // first point with at least j+1 eigenvalues below it
    const double xf = __shfl_sync(0xffffffffu, x, f);
    const double xl = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
    hi = xf;
    if (f > 0) lo = xl;
  }
  if (lane == 0) s.lam[j] = 0.5 * (lo + hi);
}

__device__ __forceinline__ double rr_start_value(int j, int i)
{
  unsigned long long z = 0x9E3779B97F4A7C15ull * (unsigned long long)(j * 1031 + i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// 5. inverse iteration for eigenvalue j: Gaussian elimination with partial
// pivoting of T - lambda I (upper factor with two superdiagonals), three
// solves from a pseudo-random start; vector j into s.X (ld m)
__global__ void __launch_bounds__(32) rr_invit_kernel(int m, rr_scratch s)
{
  __shared__ double u0i[RR_MAX_M], u1[RR_MAX_M], u2[RR_MAX_M], mu[RR_MAX_M], y[RR_MAX_M];
  __shared__ unsigned char sw[RR_MAX_M];
  __shared__ int bad;
  if (s.status[0]) return;
  const int lane = threadIdx.x, j = blockIdx.x;
  const double lam = s.lam[j];
  if (lane == 0) {
    double tn = 0.0;
    for (int i = 0; i < m; i++)
      tn = fmax(tn, fabs(s.d[i]) + (i > 0 ? fabs(s.e[i - 1]) : 0.0) + (i + 1 < m ? fabs(s.e[i]) : 0.0));
    const double tiny = DBL_EPSILON * fmax(tn, 1e-280);
    double p0 = s.d[0] - lam, p1 = m > 1 ? s.e[0] : 0.0;
    for (int k = 0; k + 1 < m; k++) {
      const double b = s.e[k], a1 = s.d[k + 1] - lam, c1 = (k + 2 < m) ? s.e[k + 1] : 0.0;
      if (fabs(p0) >= fabs(b)) {
        if (fabs(p0) < tiny) p0 = p0 < 0.0 ? -tiny : tiny;
        const double f = b / p0;
        u0i[k] = 1.0 / p0;
        u1[k] = p1;
        u2[k] = 0.0;
        mu[k] = f;
        sw[k] = 0;
        p0 = a1 - f * p1;
        p1 = c1;
      } else {
        const double f = p0 / b;
        u0i[k] = 1.0 / b;
        u1[k] = a1;
        u2[k] = c1;
        mu[k] = f;
        sw[k] = 1;
        p0 = p1 - f * a1;
        p1 = -f * c1;
      }
    }
    if (fabs(p0) < tiny) p0 = p0 < 0.0 ? -tiny : tiny;
    u0i[m - 1] = 1.0 / p0;
    bad = 0;
  }
  for (int i = lane; i < m; i += 32) y[i] = rr_start_value(j, i);
  for (int it = 0; it < 3; it++) {
    __syncwarp();
    if (lane == 0) {
      for (int k = 0; k + 1 < m; k++) {
        if (sw[k]) {
          const double t = y[k];
          y[k] = y[k + 1];
          y[k + 1] = t - mu[k] * y[k];
        } else {
          y[k + 1] -= mu[k] * y[k];
        }
      }
      y[m - 1] *= u0i[m - 1];
      if (m > 1) y[m - 2] = (y[m - 2] - u1[m - 2] * y[m - 1]) * u0i[m - 2];
      for (int k = m - 3; k >= 0; k--) y[k] = (y[k] - u1[k] * y[k + 1] - u2[k] * y[k + 2]) * u0i[k];
    }
    __syncwarp();
    double mx = 0.0;
    for (int i = lane; i < m; i += 32) mx = fmax(mx, fabs(y[i]));
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (!(mx > 0.0) || !isfinite(mx)) {
      if (lane == 0) bad = 1;
      break;
    }
    double ss = 0.0;
    for (int i = lane; i < m; i += 32) {
      const double t = y[i] / mx;
      y[i] = t;
      ss += t * t;
    }
    ss = rr_warp_sum(ss);
    const double inv = 1.0 / sqrt(ss);
    for (int i = lane; i < m; i += 32) y[i] *= inv;
  }
  __syncwarp();
  if (bad) {
    if (lane == 0) s.status[0] = 6;
    return;
  }
  for (int i = lane; i < m; i += 32) s.X[i + (size_t)j * m] = y[i];
}

// Cholesky of the nev x nev Gram matrix s.S (upper, U'U = S) and U^-1 into
// s.P; status 6 when the vectors are not numerically independent
__global__ void __launch_bounds__(256) rr_cholinv_kernel(int nev, rr_scratch s)
{
  __shared__ int bad;
  if (s.status[0]) return;
  double* U = s.S;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < nev; j++) {
    if (tid == 0) {
      const double djj = U[j + (size_t)j * nev];
      if (!(djj > 1e-6)) bad = 1;  // the vectors are unit vectors
      else U[j + (size_t)j * nev] = sqrt(djj);
    }
    __syncthreads();
    if (bad) break;
    const double r = 1.0 / U[j + (size_t)j * nev];
    for (int c = j + 1 + tid; c < nev; c += nt) U[j + (size_t)c * nev] *= r;
    __syncthreads();
    const int w = nev - j - 1;
    for (int e = tid; e < w * w; e += nt) {
      const int a = j + 1 + e % w, c = j + 1 + e / w;
      if (a <= c) U[a + (size_t)c * nev] -= U[j + (size_t)a * nev] * U[j + (size_t)c * nev];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) s.status[0] = 6;
    return;
  }
  // inverse of the upper factor, one thread per column
  for (int c = tid; c < nev; c += nt) {
    double* x = s.P + (size_t)c * nev;
    for (int i = nev - 1; i > c; i--) x[i] = 0.0;
    x[c] = 1.0 / U[c + (size_t)c * nev];
    for (int i = c - 1; i >= 0; i--) {
      double t = 0.0;
      for (int l = i + 1; l <= c; l++) t += U[i + (size_t)l * nev] * x[l];
      x[i] = -t / U[i + (size_t)i * nev];
    }
  }
}

// 6. z <- H_0 H_1 ... H_{m-3} z for the nev vectors of s.X, one warp (one
// CTA) per vector, SL = ceil(m / 32) register slots
template <int SL>
__global__ void __launch_bounds__(32) rr_backtr_kernel(int m, int nev, rr_scratch s)
{
  if (s.status[0]) return;
  const int lane = threadIdx.x;
  const int j = blockIdx.x;
  if (j >= nev) return;
  double z[SL];
  double* zc = s.X + (size_t)j * m;
#pragma unroll
  for (int q = 0; q < SL; q++) {
    const int i = q * 32 + lane;
    z[q] = i < m ? zc[i] : 0.0;
  }
  for (int h = m - 3; h >= 0; h--) {
    const double tau = s.tau[h];
    if (tau == 0.0) continue;
    const double* vh = s.C64 + (size_t)h * m;  // v(h+1) = 1, v(i) = C[i, h] for i >= h+2
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < SL; q++) {
      const int i = q * 32 + lane;
      if (i == h + 1)
        t += z[q];
      else if (i > h + 1 && i < m)
        t += vh[i] * z[q];
    }
    t = tau * rr_warp_sum(t);
#pragma unroll
    for (int q = 0; q < SL; q++) {
      const int i = q * 32 + lane;
      if (i == h + 1)
        z[q] -= t;
      else if (i > h + 1 && i < m)
        z[q] -= t * vh[i];
    }
  }
#pragma unroll
  for (int q = 0; q < SL; q++) {
    const int i = q * 32 + lane;
    if (i < m) zc[i] = z[q];
  }
}

// launch with the register slots m needs (m <= RR_MAX_M)
#define RR_SL_CASES(F) \
  F(1) F(2) F(3) F(4) F(5) F(6) F(7) F(8) F(9) F(10) F(11) F(12)
static void rr_trsm(cudaStream_t st, int mode, const double* Y, int ldy, double* X, int ldx, int m,
                    int ncols, const rr_scratch& s)
{
  switch ((m + 31) / 32) {
#define RR_TRSM_CASE(n) \
  case n: rr_trsm64_kernel<n><<<ncols, 32, 0, st>>>(mode, Y, ldy, X, ldx, m, ncols, s); break;
    RR_SL_CASES(RR_TRSM_CASE)
#undef RR_TRSM_CASE
  }
}

static void rr_backtr(cudaStream_t st, int m, int nev, const rr_scratch& s)
{
  switch ((m + 31) / 32) {
#define RR_BACKTR_CASE(n) \
  case n: rr_backtr_kernel<n><<<nev, 32, 0, st>>>(m, nev, s); break;
    RR_SL_CASES(RR_BACKTR_CASE)
#undef RR_BACKTR_CASE
  }
}
static_assert(RR_MAX_M <= 12 * 32, "rr_trsm / rr_backtr cases cover m <= 384");

// gated FP64 fallback (dense.cu)
extern "C" int gb_sygv_fp64(gpu_Context* ctx, double* A, double* B, int ld, int m, double* w,
                            int* info, const int* gate, int force);

static char* rr_take(char* base, size_t* off, size_t b)
{
  char* p = base + *off;
  *off += (b + 255) / 256 * 256;
  return p;
}

static int rr_scratch_setup(gpu_Context* ctx, int m, rr_scratch* s)
{
  const size_t mm = (size_t)m * m;
  const size_t bytes = 2 * mm * sizeof(float) + 512 * sizeof(float) + 16 * mm * sizeof(double) +
                       4 * 512 * sizeof(double) + 64 + 24 * 256;
  char* base = (char*)gb_workspace(ctx, bytes);
  if (!base) return -1;
  size_t off = 0;
  s->C = (float*)rr_take(base, &off, mm * 4);
  s->V = (float*)rr_take(base, &off, mm * 4);
  s->lam32 = (float*)rr_take(base, &off, 512 * 4);
  double** f64[] = {&s->L64, &s->LT64, &s->C64, &s->W64, &s->X, &s->Xn, &s->TA, &s->S,
                    &s->P,   &s->EI,   &s->Q,   &s->F,   &s->J1, &s->J2};
  for (size_t i = 0; i < sizeof(f64) / sizeof(f64[0]); i++) *f64[i] = (double*)rr_take(base, &off, mm * 8);
  s->lam = (double*)rr_take(base, &off, 512 * 8);
  s->d = (double*)rr_take(base, &off, 512 * 8);
  s->e = (double*)rr_take(base, &off, 512 * 8);
  s->tau = (double*)rr_take(base, &off, 512 * 8);
  s->status = (int*)rr_take(base, &off, 64);
  s->count = ctx->dcount;
  return 0;
}

#define RR_STAGE(cls, flops, launch) \
  gb_prof_begin(ctx, &ps, cls);      \
  launch;                            \
  gb_prof_end(ctx, &ps, 8.0 * m * m, flops)

// steps 1-2 (shared by both paths): L, C = inv(L) A inv(L)' symmetrised
static void rr_reduce(gpu_Context* ctx, double* A, double* B, int ld, int m, int* info,
                      rr_scratch& s, int jacobi32, double report_below)
{
  cudaStream_t st = S_(ctx);
  gb_prof_rec ps;
  const double m3 = (double)m * m * m;
  const size_t mm = (size_t)m * m;
  if (m <= RR_CHOL_SMEM_M) {
    const int sm = (int)(sizeof(double) * (size_t)m * m);
    cudaFuncSetAttribute(rr_chol64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    RR_STAGE(GB_K_RR_CHOL, m3 / 3,
             (rr_chol64_kernel<true><<<1, RR_THREADS, sm, st>>>(B, ld, m, s, info, report_below)));
  } else {
    RR_STAGE(GB_K_RR_CHOL, m3 / 3,
             (rr_chol64_kernel<false><<<1, RR_THREADS, 0, st>>>(B, ld, m, s, info, report_below)));
  }
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm(st, 0, A, ld, s.W64, m, m, m, s)));
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm(st, 1, s.W64, m, s.C64, m, m, m, s)));
  if (jacobi32) rr_sym_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(m, s);
  rr_sym_store_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(m, s);
  gb_count_launch(4 + jacobi32);
}

static void rr_tridiag_path(gpu_Context* ctx, double* A, int ld, int m, int nev, double* w,
                            int* info, rr_scratch& s)
{
  cudaStream_t st = S_(ctx);
  gb_prof_rec ps;
  const double m3 = (double)m * m * m;
  if (m <= RR_TRD_SMEM_M) {
    const int sm = (int)(sizeof(double) * (size_t)m * (m + 1) / 2);
    cudaFuncSetAttribute(rr_tridiag_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    RR_STAGE(GB_K_RR_TRID, 4.0 * m3 / 3.0,
             (rr_tridiag_smem_kernel<<<1, RR_TRD_THREADS, sm, st>>>(m, s)));
  } else {
    RR_STAGE(GB_K_RR_TRID, 4.0 * m3 / 3.0, (rr_tridiag_kernel<<<1, RR_TRD_THREADS, 0, st>>>(m, s)));
  }
  RR_STAGE(GB_K_RR_EIG, 0.0, (rr_bisect_kernel<<<nev, 32, 0, st>>>(m, s)));
  RR_STAGE(GB_K_RR_EIG, 0.0, (rr_invit_kernel<<<nev, 32, 0, st>>>(m, s)));
  // Cholesky-QR twice: Z <- Z inv(U), U'U = Z'Z
  const dim3 gs((nev + 31) / 32, (nev + 31) / 32, 1), gz((m + 31) / 32, (nev + 31) / 32, 1);
  for (int round = 0; round < 2; round++) {
    rr_gemm_t zz = {s.X, m, 1, s.X, m, s.S, nev, nev, nev, m};
    RR_STAGE(GB_K_RR_GEMM, 2.0 * m * nev * nev, (rr_gemm_kernel<<<gs, 256, 0, st>>>(zz, zz, s.status)));
    RR_STAGE(GB_K_RR_EIG, 0.0, (rr_cholinv_kernel<<<1, 256, 0, st>>>(nev, s)));
    rr_gemm_t zu = {s.X, m, 0, s.P, nev, s.Xn, m, m, nev, nev};
    RR_STAGE(GB_K_RR_GEMM, 2.0 * m * nev * nev, (rr_gemm_kernel<<<gz, 256, 0, st>>>(zu, zu, s.status)));
    double* t = s.X;
    s.X = s.Xn;
    s.Xn = t;
  }
  RR_STAGE(GB_K_RR_TRSM, 2.0 * m * m * nev, (rr_backtr(st, m, nev, s)));
  RR_STAGE(GB_K_RR_TRSM, (double)m * m * nev,
           (rr_trsm(st, 2, s.X, m, A, ld, m, nev, s)));
  rr_finish_kernel<<<(unsigned)((nev + 255) / 256), 256, 0, st>>>(nev, s, w, info);
  gb_count_launch(12);
}

static void rr_jacobi32_path(gpu_Context* ctx, double* A, int ld, int m, int nev, double* w,
                             int* info, rr_scratch& s)
{
  cudaStream_t st = S_(ctx);
  gb_prof_rec ps;
  const double m3 = (double)m * m * m;
  // Jacobi: every CTA holds C (m*m) and `rows` rows of V
  const int nsplit = m <= 96 ? 1 : 4;
  const int rows = (m + nsplit - 1) / nsplit;
  const size_t sm_jac = ((size_t)m * rr_pad(m) + (size_t)rows * rr_pad(m)) * sizeof(float);
  cudaFuncSetAttribute(rr_jacobi32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_jac);
  RR_STAGE(GB_K_RR_JAC32, 0.0, (rr_jacobi32_kernel<<<nsplit, RR_THREADS, sm_jac, st>>>(m, rows, s)));
  rr_vsort_kernel<<<1, RR_THREADS, 0, st>>>(m, s);
  int launches = 2;
  const size_t sm_ref = 2 * sizeof(double) * RR_CLUSTER_SMEM * rr_pad(RR_CLUSTER_SMEM);
  cudaFuncSetAttribute(rr_refine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_ref);
  const dim3 g1((m + 31) / 32, (m + 31) / 32, 1), g2((m + 31) / 32, (m + 31) / 32, 2);
  for (int round = 0; round < 2; round++) {
    rr_gemm_t ta = {s.C64, m, 0, s.X, m, s.TA, m, m, m, m};  // C X
    RR_STAGE(GB_K_RR_GEMM, 2 * m3, (rr_gemm_kernel<<<g1, 256, 0, st>>>(ta, ta, s.status)));
    rr_gemm_t sa = {s.X, m, 1, s.TA, m, s.S, m, m, m, m};  // X' C X
    rr_gemm_t sb = {s.X, m, 1, s.X, m, s.P, m, m, m, m};   // X' X
    RR_STAGE(GB_K_RR_GEMM, 4 * m3, (rr_gemm_kernel<<<g2, 256, 0, st>>>(sa, sb, s.status)));
    RR_STAGE(GB_K_RR_REFINE, 0.0, (rr_refine_kernel<<<1, RR_THREADS, sm_ref, st>>>(m, s, round == 1)));
    rr_gemm_t fq = {s.EI, m, 0, s.Q, m, s.F, m, m, m, m};
    RR_STAGE(GB_K_RR_GEMM, 2 * m3, (rr_gemm_kernel<<<g1, 256, 0, st>>>(fq, fq, s.status)));
    rr_gemm_t xf = {s.X, m, 0, s.F, m, s.Xn, m, m, m, m};
    RR_STAGE(GB_K_RR_GEMM, 2 * m3, (rr_gemm_kernel<<<g1, 256, 0, st>>>(xf, xf, s.status)));
    double* t = s.X;
    s.X = s.Xn;
    s.Xn = t;
    launches += 5;
  }
  // eigenvectors of the pencil: inv(L)' X into A; values into w
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm(st, 2, s.X, m, A, ld, m, m, s)));
  rr_finish_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(nev, s, w, info);
  gb_count_launch(launches + 2);
}
#undef RR_STAGE

extern "C" int gb_sygv(gpu_Context* ctx, double* A, double* B, int ld, int m, int nev, double* w,
                       int* info, double report_below)
{
  ctx->sygv_calls++;
  const int forced = ctx->opt.sygv_fail_at > 0 && ctx->sygv_calls == ctx->opt.sygv_fail_at;
  const int method = ctx->opt.rr_method;
  if (nev < 1 || nev > m) nev = m;
  if (forced || m < 2 || m > RR_MAX_M || method == 1 || (method == 2 && m > RR_MAX_SMEM_M))
    return gb_sygv_fp64(ctx, A, B, ld, m, w, info, NULL, forced);
  rr_scratch s;
  if (rr_scratch_setup(ctx, m, &s)) return -1;
  gb_prof_rec pr;
  const double m3 = (double)m * m * m;
  gb_prof_begin(ctx, &pr, GB_K_SYGV);
  rr_reduce(ctx, A, B, ld, m, info, s, method == 2, report_below);
  if (method == 2)
    rr_jacobi32_path(ctx, A, ld, m, nev, w, info, s);
  else
    rr_tridiag_path(ctx, A, ld, m, nev, w, info, s);
  gb_prof_end(ctx, &pr, 32.0 * m * m, 4.0 * m3);
  if (gb_cuda_check(ctx, (int)cudaGetLastError(), "rayleigh_ritz")) return -1;
  // FP64 Jacobi on the original pencil when the fast path did not finish
  return gb_sygv_fp64(ctx, A, B, ld, m, w, info, s.status, 0);
}
