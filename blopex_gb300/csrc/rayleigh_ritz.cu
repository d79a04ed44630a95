// rayleigh_ritz.cu -- the Rayleigh-Ritz eigenproblem A v = w B v (B SPD,
// order m <= 3k) of every LOBPCG iteration, replacing the dsygv call of
// lobpcg_solveGEVP (blopex_abstract/krylov/lobpcg.c:66-103), built for a GPU
// whose FP32 rate is 64 times its FP64 rate:
//
//   1. FP32, one CTA: Cholesky B = L L', C = inv(L) A inv(L)'          (rr_reduce32)
//   2. FP32, cyclic Jacobi on C; every CTA rotates its own copy of C
//      (identical arithmetic, no communication) and accumulates its own
//      slice of rows of the eigenvector matrix V                       (rr_jacobi32)
//   3. FP32, X = inv(L)' V sorted by eigenvalue, widened to FP64         (rr_backsub32)
//   4. FP64 refinement of the eigenvector matrix, twice: with
//      S = X'AX and P = X'BX (multi-CTA FP64 GEMMs), the Ritz values
//      l_i = S_ii / P_ii and the correction X <- X (I + E),
//        E_ij = (S_ij - l_j P_ij) / (l_j - l_i)   for separated pairs,
//        E_ij = R_ij / 2 with R = I - P           inside clusters,
//      and inside each cluster of close values the FP64 matrix
//      S_cc + (R_cc S_cc + S_cc R_cc)/2 is diagonalised by FP64 Jacobi.
//      This is the iterative refinement of Ogita & Aishima (symmetric
//      eigenproblems, Japan J. Indust. Appl. Math. 2018) written for the
//      B-inner product; each round squares the eigenvector error.
//   5. the first m columns of X and the values go to A and w (dsygv's
//      outputs; B is left intact).
// If the FP32 Cholesky or Jacobi fails, the one-CTA FP64 Jacobi solver of
// dense.cu runs instead (gated on a device status word, no host sync).
// Every loop has a fixed trip count.
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
  float *L, *C, *W, *V, *lam32;
  double *X, *Xn, *TA, *TB, *S, *P, *EI, *Q, *F, *J1, *J2, *lam;
  int* status;
};

// ------------------------------------------------------------------ 1.
__global__ void __launch_bounds__(RR_THREADS) rr_reduce32_kernel(const double* __restrict__ A,
                                                                 const double* __restrict__ B,
                                                                 int ld, int m, rr_scratch s)
{
  extern __shared__ float Ls[];  // m*m, column-major
  __shared__ int bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) {
    bad = 0;
    s.status[0] = 0;
  }
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    Ls[e] = (i >= j) ? (float)B[i + (size_t)j * ld] : 0.f;
  }
  __syncthreads();
  // right-looking Cholesky, lower
  for (int j = 0; j < m; j++) {
    if (tid == 0) {
      float d = Ls[j + j * m];
      if (!(d > 0.f) || !isfinite(d))
        bad = 1;
      else
        Ls[j + j * m] = sqrtf(d);
    }
    __syncthreads();
    if (bad) break;
    const float djj = Ls[j + j * m];
    for (int i = j + 1 + tid; i < m; i += nt) Ls[i + j * m] /= djj;
    __syncthreads();
    const int r = m - j - 1;
    for (int e = tid; e < r * r; e += nt) {
      int i = j + 1 + e % r, l = j + 1 + e / r;
      if (i >= l) Ls[i + l * m] -= Ls[i + j * m] * Ls[l + j * m];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) s.status[0] = 1;
    return;
  }
  for (int e = tid; e < m * m; e += nt) s.L[e] = Ls[e];
  // W = inv(L) A, one thread per column, A symmetric from its lower triangle
  for (int j = tid; j < m; j += nt) {
    float* w = s.W + (size_t)j * m;
    for (int i = 0; i < m; i++) {
      float a = (float)((i >= j) ? A[i + (size_t)j * ld] : A[j + (size_t)i * ld]);
      for (int p = 0; p < i; p++) a -= Ls[i + p * m] * w[p];
      w[i] = a / Ls[i + i * m];
    }
  }
  __syncthreads();
  // C = inv(L) W' (column j of C solves L c = row j of W)
  for (int j = tid; j < m; j += nt) {
    float* c = s.C + (size_t)j * m;
    for (int i = 0; i < m; i++) {
      float a = s.W[j + (size_t)i * m];
      for (int p = 0; p < i; p++) a -= Ls[i + p * m] * c[p];
      c[i] = a / Ls[i + i * m];
    }
  }
  __syncthreads();
  for (int e = tid; e < m * m; e += nt) {
    int i = e % m, j = e / m;
    if (i > j) {
      float v = 0.5f * (s.C[i + (size_t)j * m] + s.C[j + (size_t)i * m]);
      s.C[i + (size_t)j * m] = v;
      s.C[j + (size_t)i * m] = v;
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

__global__ void __launch_bounds__(RR_THREADS) rr_jacobi32_kernel(int m, int rows, rr_scratch s)
{
  extern __shared__ float sm[];
  float* Cs = sm;            // m*m
  float* Vs = sm + m * m;    // rows*m: rows r0..r0+rows of V, row-major by V row
  __shared__ float s_c[256], s_s[256];
  __shared__ int s_p[256], s_q[256];
  __shared__ int s_done;
  __shared__ float s_red[RR_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int r0 = blockIdx.x * rows;
  const int nr = min(rows, m - r0);
  if (s.status[0]) return;
  for (int e = tid; e < m * m; e += nt) Cs[e] = s.C[e];
  for (int e = tid; e < rows * m; e += nt) {
    int r = e / m, c = e % m;
    Vs[e] = (r0 + r == c) ? 1.f : 0.f;
  }
  float acc = 0.f;
  for (int e = tid; e < m * m; e += nt) acc += Cs[e] * Cs[e];
  s_red[tid] = acc;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) s_red[tid] += s_red[tid + o];
    __syncthreads();
  }
  const float nrm = sqrtf(s_red[0]);
  const float thr_rot = 0.05f * FLT_EPSILON * nrm;
  const float thr_done = 8.f * FLT_EPSILON * nrm;
  const int me = (m + 1) & ~1, half = me / 2;
  int converged = 0, sweep = 0;
  for (; sweep < JACOBI32_MAX_SWEEPS && !converged; sweep++) {
    if (tid == 0) s_done = 1;
    __syncthreads();
    for (int round = 0; round < me - 1; round++) {
      for (int t = tid; t < half; t += nt) {
        int p, q;
        rr_pair(t, round, me, &p, &q);
        float c = 1.f, sn = 0.f;
        if (q < m) {
          float apq = Cs[p + q * m], app = Cs[p + p * m], aqq = Cs[q + q * m];
          if (fabsf(apq) > thr_rot) {
            float theta = (aqq - app) / (2.f * apq);
            float tt = (theta >= 0.f ? 1.f : -1.f) / (fabsf(theta) + sqrtf(1.f + theta * theta));
            c = rsqrtf(1.f + tt * tt);
            sn = tt * c;
            if (fabsf(apq) > thr_done) s_done = 0;
          }
        }
        s_p[t] = p;
        s_q[t] = q;
        s_c[t] = c;
        s_s[t] = sn;
      }
      __syncthreads();
      for (int e = tid; e < half * m; e += nt) {
        int t = e / m, j = e % m;
        float sn = s_s[t];
        if (sn == 0.f) continue;
        int p = s_p[t], q = s_q[t];
        float c = s_c[t];
        float ap = Cs[p + j * m], aq = Cs[q + j * m];
        Cs[p + j * m] = c * ap - sn * aq;
        Cs[q + j * m] = sn * ap + c * aq;
      }
      __syncthreads();
      for (int e = tid; e < half * m; e += nt) {
        int t = e / m, i = e % m;
        float sn = s_s[t];
        if (sn == 0.f) continue;
        int p = s_p[t], q = s_q[t];
        float c = s_c[t];
        float ap = Cs[i + p * m], aq = Cs[i + q * m];
        Cs[i + p * m] = c * ap - sn * aq;
        Cs[i + q * m] = sn * ap + c * aq;
      }
      for (int e = tid; e < half * nr; e += nt) {
        int t = e / nr, r = e % nr;
        float sn = s_s[t];
        if (sn == 0.f) continue;
        int p = s_p[t], q = s_q[t];
        float c = s_c[t];
        float vp = Vs[r * m + p], vq = Vs[r * m + q];
        Vs[r * m + p] = c * vp - sn * vq;
        Vs[r * m + q] = sn * vp + c * vq;
      }
      __syncthreads();
      for (int t = tid; t < half; t += nt)
        if (s_s[t] != 0.f) {
          Cs[s_p[t] + s_q[t] * m] = 0.f;
          Cs[s_q[t] + s_p[t] * m] = 0.f;
        }
      __syncthreads();
    }
    converged = s_done;
    __syncthreads();
  }
  if (!converged) {
    if (tid == 0) s.status[0] = 2;
    return;
  }
  for (int e = tid; e < nr * m; e += nt) {
    int r = e / m, c = e % m;
    s.V[(r0 + r) + (size_t)c * m] = Vs[r * m + c];
  }
  if (blockIdx.x == 0) {
    for (int i = tid; i < m; i += nt) s.lam32[i] = Cs[i + i * m];
    if (tid == 0) s.status[1] = sweep;
  }
}

// ------------------------------------------------------------------ 3.
__global__ void __launch_bounds__(RR_THREADS) rr_backsub32_kernel(int m, rr_scratch s)
{
  extern __shared__ float Ls[];
  __shared__ int perm[512];
  const int tid = threadIdx.x, nt = blockDim.x;
  if (s.status[0]) return;
  for (int e = tid; e < m * m; e += nt) Ls[e] = s.L[e];
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
  // x = inv(L)' v, one thread per output column; accumulate in FP32 then widen
  for (int r = tid; r < m; r += nt) {
    const float* v = s.V + (size_t)perm[r] * m;
    double* x = s.X + (size_t)r * m;
    float* tmp = s.W + (size_t)r * m;  // W is free scratch now
    for (int i = m - 1; i >= 0; i--) {
      float a = v[i];
      for (int p = i + 1; p < m; p++) a -= Ls[p + i * m] * tmp[p];
      tmp[i] = a / Ls[i + i * m];
      x[i] = (double)tmp[i];
    }
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

// FP64 cyclic Jacobi on the c x c matrix M (ld c) with eigenvectors in V,
// all threads of the block; returns 1 when converged.
__device__ int rr_jacobi64(double* M, double* V, int c)
{
  __shared__ double j_c[256], j_s[256];
  __shared__ int j_p[256], j_q[256];
  __shared__ int j_done;
  __shared__ double j_red[RR_THREADS];
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < c * c; e += nt) V[e] = (e % c == e / c) ? 1.0 : 0.0;
  double acc = 0.0;
  for (int e = tid; e < c * c; e += nt) acc += M[e] * M[e];
  j_red[tid] = acc;
  __syncthreads();
  for (int o = nt / 2; o > 0; o >>= 1) {
    if (tid < o) j_red[tid] += j_red[tid + o];
    __syncthreads();
  }
  const double nrm = sqrt(j_red[0]);
  const double thr_rot = 1e-3 * DBL_EPSILON * nrm, thr_done = 4.0 * DBL_EPSILON * nrm;
  const int me = (c + 1) & ~1, half = me / 2;
  int converged = 0;
  for (int sweep = 0; sweep < JACOBI64_MAX_SWEEPS && !converged; sweep++) {
    if (tid == 0) j_done = 1;
    __syncthreads();
    for (int round = 0; round < me - 1; round++) {
      for (int t = tid; t < half; t += nt) {
        int p, q;
        rr_pair(t, round, me, &p, &q);
        double cs = 1.0, sn = 0.0;
        if (q < c) {
          double apq = M[p + q * c], app = M[p + p * c], aqq = M[q + q * c];
          if (fabs(apq) > thr_rot) {
            double theta = (aqq - app) / (2.0 * apq);
            double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(1.0 + theta * theta));
            cs = 1.0 / sqrt(1.0 + tt * tt);
            sn = tt * cs;
            if (fabs(apq) > thr_done) j_done = 0;
          }
        }
        j_p[t] = p;
        j_q[t] = q;
        j_c[t] = cs;
        j_s[t] = sn;
      }
      __syncthreads();
      for (int e = tid; e < half * c; e += nt) {
        int t = e / c, j = e % c;
        double sn = j_s[t];
        if (sn == 0.0) continue;
        int p = j_p[t], q = j_q[t];
        double cs = j_c[t];
        double ap = M[p + j * c], aq = M[q + j * c];
        M[p + j * c] = cs * ap - sn * aq;
        M[q + j * c] = sn * ap + cs * aq;
      }
      __syncthreads();
      for (int e = tid; e < half * c; e += nt) {
        int t = e / c, i = e % c;
        double sn = j_s[t];
        if (sn == 0.0) continue;
        int p = j_p[t], q = j_q[t];
        double cs = j_c[t];
        double ap = M[i + p * c], aq = M[i + q * c];
        M[i + p * c] = cs * ap - sn * aq;
        M[i + q * c] = sn * ap + cs * aq;
        double vp = V[i + p * c], vq = V[i + q * c];
        V[i + p * c] = cs * vp - sn * vq;
        V[i + q * c] = sn * vp + cs * vq;
      }
      __syncthreads();
      for (int t = tid; t < half; t += nt)
        if (j_s[t] != 0.0) {
          M[j_p[t] + j_q[t] * c] = 0.0;
          M[j_q[t] + j_p[t] * c] = 0.0;
        }
      __syncthreads();
    }
    converged = j_done;
    __syncthreads();
  }
  return converged;
}

// refinement step: S = X'AX, P = X'BX -> EI = I + E, Q (block diagonal on
// the clusters), lam
__global__ void __launch_bounds__(RR_THREADS) rr_refine_kernel(int m, rr_scratch s, int last)
{
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
  const double delta = 1e-3 * s_red[0] + 1e-300;
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
    double* Mc = s.J1;
    double* Vc = s.J2;
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      double v = S[(a0 + a) + (size_t)(a0 + b) * m];
      double t = 0.0;
      for (int l = 0; l < sz; l++) {
        double ral = (a == l ? 1.0 : 0.0) - P[(a0 + a) + (size_t)(a0 + l) * m];
        double rlb = (l == b ? 1.0 : 0.0) - P[(a0 + l) + (size_t)(a0 + b) * m];
        t += ral * S[(a0 + l) + (size_t)(a0 + b) * m] + S[(a0 + a) + (size_t)(a0 + l) * m] * rlb;
      }
      Mc[a + b * sz] = v + 0.5 * t;
    }
    __syncthreads();
    // symmetrise
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, b = e / sz;
      if (a > b) {
        double v = 0.5 * (Mc[a + b * sz] + Mc[b + a * sz]);
        Mc[a + b * sz] = v;
        Mc[b + a * sz] = v;
      }
    }
    __syncthreads();
    int ok = rr_jacobi64(Mc, Vc, sz);
    if (!ok) {
      if (tid == 0) s.status[0] = 3;
      return;
    }
    // ascending order inside the cluster
    __shared__ int cperm[512];
    for (int a = tid; a < sz; a += nt) {
      double da = Mc[a + a * sz];
      int r = 0;
      for (int b = 0; b < sz; b++) {
        double db = Mc[b + b * sz];
        if (db < da || (db == da && b < a)) r++;
      }
      cperm[r] = a;
    }
    __syncthreads();
    for (int e = tid; e < sz * sz; e += nt) {
      int a = e % sz, r = e / sz;
      s.Q[(a0 + a) + (size_t)(a0 + r) * m] = Vc[a + cperm[r] * sz];
    }
    for (int r = tid; r < sz; r += nt) s.lam[a0 + r] = Mc[cperm[r] + cperm[r] * sz];
    __syncthreads();
  }
}

__global__ void rr_finish_kernel(int m, rr_scratch s, double* A, int ld, double* w, int* info)
{
  if (s.status[0]) return;  // the FP64 fallback writes the outputs
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
    int i = e % m, j = e / m;
    A[i + (size_t)j * ld] = s.X[e];
  }
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
  size_t bytes = 4 * mm * sizeof(float) + 512 * sizeof(float) + 13 * mm * sizeof(double) +
                 512 * sizeof(double) + 64;
  char* base = (char*)gb_workspace(ctx, bytes + 1024);
  if (!base) return -1;
  rr_scratch s;
  size_t off = 0;
  auto take = [&](size_t b) {
    char* p = base + off;
    off += (b + 255) / 256 * 256;
    return p;
  };
  s.L = (float*)take(mm * 4);
  s.C = (float*)take(mm * 4);
  s.W = (float*)take(mm * 4);
  s.V = (float*)take(mm * 4);
  s.lam32 = (float*)take(512 * 4);
  s.X = (double*)take(mm * 8);
  s.Xn = (double*)take(mm * 8);
  s.TA = (double*)take(mm * 8);
  s.TB = (double*)take(mm * 8);
  s.S = (double*)take(mm * 8);
  s.P = (double*)take(mm * 8);
  s.EI = (double*)take(mm * 8);
  s.Q = (double*)take(mm * 8);
  s.F = (double*)take(mm * 8);
  s.J1 = (double*)take(mm * 8);
  s.J2 = (double*)take(mm * 8);
  s.lam = (double*)take(512 * 8);
  s.status = (int*)take(64);

  cudaStream_t st = S_(ctx);
  gb_prof_rec pr;
  gb_prof_begin(ctx, &pr, GB_K_SYGV);
  const size_t sm_red = mm * sizeof(float);
  cudaFuncSetAttribute(rr_reduce32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_red);
  rr_reduce32_kernel<<<1, RR_THREADS, sm_red, st>>>(A, B, ld, m, s);
  // Jacobi: every CTA holds C (m*m) and `rows` rows of V
  const int nsplit = m <= 96 ? 1 : 4;
  const int rows = (m + nsplit - 1) / nsplit;
  const size_t sm_jac = (mm + (size_t)rows * m) * sizeof(float);
  cudaFuncSetAttribute(rr_jacobi32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_jac);
  rr_jacobi32_kernel<<<nsplit, RR_THREADS, sm_jac, st>>>(m, rows, s);
  cudaFuncSetAttribute(rr_backsub32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_red);
  rr_backsub32_kernel<<<1, RR_THREADS, sm_red, st>>>(m, s);
  int launches = 3;
  const dim3 gg((m + 31) / 32, (m + 31) / 32, 2), g1((m + 31) / 32, (m + 31) / 32, 1);
  for (int round = 0; round < 2; round++) {
    rr_gemm_t ta = {A, ld, 2, s.X, m, s.TA, m, m, m, m};
    rr_gemm_t tb = {B, ld, 2, s.X, m, s.TB, m, m, m, m};
    rr_gemm_kernel<<<gg, 256, 0, st>>>(ta, tb, s.status);
    rr_gemm_t sa = {s.X, m, 1, s.TA, m, s.S, m, m, m, m};
    rr_gemm_t sb = {s.X, m, 1, s.TB, m, s.P, m, m, m, m};
    rr_gemm_kernel<<<gg, 256, 0, st>>>(sa, sb, s.status);
    rr_refine_kernel<<<1, RR_THREADS, 0, st>>>(m, s, round == 1);
    rr_gemm_t fq = {s.EI, m, 0, s.Q, m, s.F, m, m, m, m};
    rr_gemm_kernel<<<g1, 256, 0, st>>>(fq, fq, s.status);
    rr_gemm_t xf = {s.X, m, 0, s.F, m, s.Xn, m, m, m, m};
    rr_gemm_kernel<<<g1, 256, 0, st>>>(xf, xf, s.status);
    double* t = s.X;
    s.X = s.Xn;
    s.Xn = t;
    launches += 5;
  }
  rr_finish_kernel<<<(m * m + 255) / 256, 256, 0, st>>>(m, s, A, ld, w, info);
  launches++;
  gb_prof_end(ctx, &pr, 32.0 * m * m, 2.0 * 2.0 * 5.0 * (double)m * m * m);
  gb_count_launch(launches);
  if (gb_cuda_check(ctx, (int)cudaGetLastError(), "rayleigh_ritz")) return -1;
  // FP64 Jacobi on the original pencil when the FP32 stage failed
  return gb_sygv_fp64(ctx, A, B, ld, m, w, info, s.status, 0);
}
