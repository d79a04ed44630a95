// rayleigh_ritz.cu -- the Rayleigh-Ritz eigenproblem A v = w B v (B SPD,
// order m <= 3k) of every LOBPCG iteration, replacing the dsygv call of
// lobpcg_solveGEVP (blopex_abstract/krylov/lobpcg.c:66-103), built for a GPU
// whose FP32 rate is 64 times its FP64 rate:
//
//   1. FP64, one CTA: Cholesky B = L L' (its failure is dsygv's INFO m+j)
//   2. FP64, multi-CTA triangular solves: C = inv(L) A inv(L)'   -- the
//      conditioning of B is handled here, in FP64, as dsygv does
//   3. FP32, cyclic Jacobi on C; every CTA rotates its own copy of C
//      (identical arithmetic, no communication) and accumulates its own
//      slice of rows of the eigenvector matrix V
//   4. FP64 refinement of V, twice: with S = V'CV and P = V'V
//      (multi-CTA FP64 GEMMs), the Ritz values l_i = S_ii / P_ii and the
//      correction V <- V (I + E),
//        E_ij = (S_ij - l_j P_ij) / (l_j - l_i)   for separated pairs,
//        E_ij = R_ij / 2 with R = I - P           inside clusters,
//      and inside each cluster of close values the FP64 matrix
//      S_cc + (R_cc S_cc + S_cc R_cc)/2 is diagonalised by FP64 Jacobi.
//      This is the iterative refinement of Ogita & Aishima (symmetric
//      eigenproblems, Japan J. Indust. Appl. Math. 2018); each round
//      squares the eigenvector error.
//   5. FP64, multi-CTA: eigenvectors of the pencil inv(L)' V into A, values
//      into w (dsygv's outputs; B is left intact).
// If the FP32 Jacobi does not converge or the refinement does not settle,
// the one-CTA FP64 Jacobi solver of dense.cu runs on the original pencil
// instead (gated on a device status word, no host sync).  Every loop has a
// fixed trip count.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>

#include "internal.h"

static inline cudaStream_t S_(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

#define RR_THREADS 1024
#define RR_MAX_SMEM_M 192
#define JACOBI32_MAX_SWEEPS 30
#define JACOBI64_MAX_SWEEPS 40

// status words (device ints): [0] fast path failed, [1] Jacobi32 sweeps
struct rr_scratch {
  int* count;  // context counters (see internal.h)
  float *C, *V, *lam32;
  double *L64, *LT64, *C64, *W64;
  double *X, *Xn, *TA, *S, *P, *EI, *Q, *F, *J1, *J2, *lam;
  int* status;
};

// ------------------------------------------------------------------ 1.
// FP64 lower Cholesky of B into s.L64 (m x m, ld m); *info = m + j on
// failure (dsygv's convention for a B that is not positive definite).
__global__ void __launch_bounds__(RR_THREADS) rr_chol64_kernel(const double* __restrict__ B, int ld,
                                                               int m, rr_scratch s, int* info)
{
  __shared__ int bad;
  double* L = s.L64;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) {
    bad = 0;
    s.status[0] = 0;
  }
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    L[e] = (i >= j) ? B[i + (size_t)j * ld] : 0.0;
  }
  __syncthreads();
  for (int j = 0; j < m; j++) {
    if (tid == 0) {
      double d = L[j + (size_t)j * m];
      if (!(d > 0.0) || !isfinite(d))
        bad = j + 1;
      else
        L[j + (size_t)j * m] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    const double djj = L[j + (size_t)j * m];
    for (int i = j + 1 + tid; i < m; i += nt) L[i + (size_t)j * m] /= djj;
    __syncthreads();
    const int r = m - j - 1;
    for (int e = tid; e < r * r; e += nt) {
      int i = j + 1 + e % r, l = j + 1 + e / r;
      if (i >= l) L[i + (size_t)l * m] -= L[i + (size_t)j * m] * L[l + (size_t)j * m];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) {
      s.status[0] = 5;
      *info = m + bad;
    }
    return;
  }
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, p = e / m;
    s.LT64[p + (size_t)i * m] = L[e];
  }
}

// triangular solves with the FP64 factor, one warp per right-hand side; the
// solution lives in registers (entry p in lane p % 32, slot p / 32):
//   mode 0: X = inv(L) Y, Y symmetric read from its lower triangle (ld ldy)
//   mode 1: X = inv(L) Y' (Y m x m, ld ldy)
//   mode 2: X = inv(L)' Y (Y m x m, ld ldy), result to X with leading dim ldx
// s.LT holds L row-major (LT[p + i*m] = L(i, p)) so that the forward
// sweeps read contiguous rows of L.
#define RR_TRSM_SLOTS (RR_MAX_SMEM_M / 32)
__global__ void __launch_bounds__(256) rr_trsm64_kernel(int mode, const double* __restrict__ Y,
                                                        int ldy, double* __restrict__ X, int ldx,
                                                        int m, rr_scratch s)
{
  if (s.status[0]) return;
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= m) return;
  double xr[RR_TRSM_SLOTS];
#pragma unroll
  for (int q = 0; q < RR_TRSM_SLOTS; q++) xr[q] = 0.0;
  if (mode < 2) {
    const double* LT = s.LT64;
    for (int i = 0; i < m; i++) {
      double part = 0.0;
#pragma unroll
      for (int q = 0; q < RR_TRSM_SLOTS; q++) {
        int p = q * 32 + lane;
        if (p < i) part += LT[p + (size_t)i * m] * xr[q];
      }
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      double a;
      if (mode == 0)
        a = (i >= j) ? Y[i + (size_t)j * ldy] : Y[j + (size_t)i * ldy];
      else
        a = Y[j + (size_t)i * ldy];
      const double xi = (a - part) / LT[i + (size_t)i * m];
#pragma unroll
      for (int q = 0; q < RR_TRSM_SLOTS; q++)
        if (q * 32 + lane == i) xr[q] = xi;
    }
  } else {
    const double* L = s.L64;
    for (int i = m - 1; i >= 0; i--) {
      double part = 0.0;
#pragma unroll
      for (int q = 0; q < RR_TRSM_SLOTS; q++) {
        int p = q * 32 + lane;
        if (p > i && p < m) part += L[p + (size_t)i * m] * xr[q];
      }
      for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
      const double xi = (Y[i + (size_t)j * ldy] - part) / L[i + (size_t)i * m];
#pragma unroll
      for (int q = 0; q < RR_TRSM_SLOTS; q++)
        if (q * 32 + lane == i) xr[q] = xi;
    }
  }
  double* x = X + (size_t)j * ldx;
#pragma unroll
  for (int q = 0; q < RR_TRSM_SLOTS; q++) {
    int p = q * 32 + lane;
    if (p < m) x[p] = xr[q];
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
      atomicAdd(&s.count[3], 1);
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

__global__ void rr_finish_kernel(int m, rr_scratch s, double* w, int* info)
{
  if (s.status[0]) return;  // the FP64 fallback writes the outputs
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x)
    w[i] = s.lam[i];
  if (blockIdx.x == 0 && threadIdx.x == 0) *info = 0;
}

// gated FP64 fallback (dense.cu)
extern "C" int gb_sygv_fp64(gpu_Context* ctx, double* A, double* B, int ld, int m, double* w,
                            int* info, const int* gate, int force);

extern "C" int gb_sygv(gpu_Context* ctx, double* A, double* B, int ld, int m, double* w, int* info)
{
  ctx->sygv_calls++;
  const int forced = ctx->opt.sygv_fail_at > 0 && ctx->sygv_calls == ctx->opt.sygv_fail_at;
  if (forced || m > RR_MAX_SMEM_M || m < 2 || ctx->opt.rr_fp64_only)
    return gb_sygv_fp64(ctx, A, B, ld, m, w, info, NULL, forced);

  const size_t mm = (size_t)m * m;
  size_t bytes = 2 * mm * sizeof(float) + 512 * sizeof(float) + 16 * mm * sizeof(double) +
                 512 * sizeof(double) + 64 + 20 * 256;
  char* base = (char*)gb_workspace(ctx, bytes);
  if (!base) return -1;
  rr_scratch s;
  size_t off = 0;
  auto take = [&](size_t b) {
    char* p = base + off;
    off += (b + 255) / 256 * 256;
    return p;
  };
  s.C = (float*)take(mm * 4);
  s.V = (float*)take(mm * 4);
  s.lam32 = (float*)take(512 * 4);
  s.L64 = (double*)take(mm * 8);
  s.LT64 = (double*)take(mm * 8);
  s.C64 = (double*)take(mm * 8);
  s.W64 = (double*)take(mm * 8);
  s.X = (double*)take(mm * 8);
  s.Xn = (double*)take(mm * 8);
  s.TA = (double*)take(mm * 8);
  s.S = (double*)take(mm * 8);
  s.P = (double*)take(mm * 8);
  s.EI = (double*)take(mm * 8);
  s.Q = (double*)take(mm * 8);
  s.F = (double*)take(mm * 8);
  s.J1 = (double*)take(mm * 8);
  s.J2 = (double*)take(mm * 8);
  s.lam = (double*)take(512 * 8);
  s.status = (int*)take(64);
  s.count = ctx->dcount;

  cudaStream_t st = S_(ctx);
  gb_prof_rec pr, ps;
  gb_prof_begin(ctx, &pr, GB_K_SYGV);
  const double m3 = (double)m * m * m;
#define RR_STAGE(cls, flops, launch) \
  gb_prof_begin(ctx, &ps, cls);      \
  launch;                            \
  gb_prof_end(ctx, &ps, 8.0 * m * m, flops)
  const unsigned tb = (unsigned)((m + 7) / 8);  // 8 warps (columns) per CTA
  RR_STAGE(GB_K_RR_CHOL, m3 / 3, (rr_chol64_kernel<<<1, RR_THREADS, 0, st>>>(B, ld, m, s, info)));
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm64_kernel<<<tb, 256, 0, st>>>(0, A, ld, s.W64, m, m, s)));
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm64_kernel<<<tb, 256, 0, st>>>(1, s.W64, m, s.C64, m, m, s)));
  rr_sym_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(m, s);
  rr_sym_store_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(m, s);
  // Jacobi: every CTA holds C (m*m) and `rows` rows of V
  const int nsplit = m <= 96 ? 1 : 4;
  const int rows = (m + nsplit - 1) / nsplit;
  const size_t sm_jac = ((size_t)m * rr_pad(m) + (size_t)rows * rr_pad(m)) * sizeof(float);
  cudaFuncSetAttribute(rr_jacobi32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_jac);
  RR_STAGE(GB_K_RR_JAC32, 0.0, (rr_jacobi32_kernel<<<nsplit, RR_THREADS, sm_jac, st>>>(m, rows, s)));
  rr_vsort_kernel<<<1, RR_THREADS, 0, st>>>(m, s);
  int launches = 7;
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
  RR_STAGE(GB_K_RR_TRSM, m3, (rr_trsm64_kernel<<<tb, 256, 0, st>>>(2, s.X, m, A, ld, m, s)));
  rr_finish_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(m, s, w, info);
#undef RR_STAGE
  launches += 2;
  gb_prof_end(ctx, &pr, 32.0 * m * m, 16.0 * m3);
  gb_count_launch(launches);
  if (gb_cuda_check(ctx, (int)cudaGetLastError(), "rayleigh_ritz")) return -1;
  // FP64 Jacobi on the original pencil when the fast path did not finish
  return gb_sygv_fp64(ctx, A, B, ld, m, w, info, s.status, 0);
}
