// adjoint.cu -- reverse-mode derivatives of the computed eigenpairs (no
// counterpart in the reference, which has no derivatives).
//
// For A x_i = lambda_i B x_i with X'BX = I and a loss L(lambda, X) with
// g_lambda = dL/dlambda, G = dL/dX:
//   d lambda_i = x_i' (dA - lambda_i dB) x_i
//   d x_i      = sum_{j != i} x_j x_j'(dA - lambda_i dB) x_i / (lambda_i - lambda_j)
//                - (x_i' dB x_i) x_i / 2
// so that dL = sum_i w_i'(dA - lambda_i dB) x_i - (g_i'x_i)(x_i' dB x_i)/2 with
//   w_i = g_lambda_i x_i + mu_i,  mu_i = sum_{j != i} x_j (x_j'g_i) / (lambda_i - lambda_j).
// The sum over the k computed pairs is formed explicitly (mu_in = X M); the
// rest of the spectrum enters through mu_out, the solution of
//   (A - lambda_i B) mu = -(I - B X X') g_i,   X'B mu = 0,
// which is positive definite on the B-orthogonal complement of span(X)
// because lambda_i lies below the remaining spectrum.  It is solved by
// preconditioned conjugate gradients on the projected operator
// P_L (A - lambda_i B) P_R (P_L = I - B X X', P_R = I - X X'B), all k columns
// in lockstep (one block application of A and B per step, the projections as
// k x k Gram products and block updates).  The Polak-Ribiere form of beta
// (r_new'(z_new - z_old) / r_old'z_old, restarted when negative) keeps the
// iteration convergent when the preconditioner is itself an iteration (an
// inner CG on A).  The eigenpairs are never stored along the iteration
// history: the backward pass needs only the final X.
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdio.h>

#include "internal.h"

typedef void (*op_fn)(void*, void*, void*);

static inline cudaStream_t S(gpu_Context* ctx) { return (cudaStream_t)ctx->stream; }

// M(j, i) = S(j, i) / (lam_i - lam_j) for j != i outside degenerate pairs;
// M(i, i) = glam_i, so that X M = glam_i x_i + mu_in_i
__global__ void adj_inspace_kernel(int k, const double* __restrict__ Sg, const double* __restrict__ lam,
                                   const double* __restrict__ glam, double tol_deg, double* __restrict__ M)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= k * k) return;
  const int j = e % k, i = e / k;
  double v;
  if (i == j) {
    v = glam ? glam[i] : 0.0;
  } else {
    const double d = lam[i] - lam[j];
    v = fabs(d) > tol_deg ? Sg[j + (size_t)i * k] / d : 0.0;
  }
  M[j + (size_t)i * k] = v;
}

__global__ void adj_sub_kernel(int k, const double* a, const double* b, double* out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = a[i] - b[i];
}

__global__ void adj_neg_kernel(int m, double* A)
{
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < m) A[e] = -A[e];
}

// out_i = num_i / den_i when both are positive, else 0 (a converged column)
__global__ void adj_ratio_kernel(int k, const double* num, const double* den, double* out)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) out[i] = (num[i] > 0.0 && den[i] > 0.0) ? num[i] / den[i] : 0.0;
}

// Y_i += s a_i X_i (and Y2_i += s2 a_i X2_i when X2 is given)
__global__ void adj_axpy_cols_kernel(long n, blk_cols X, blk_cols Y, const double* a, double s,
                                     blk_cols X2, blk_cols Y2, double s2, int two)
{
  const int i = blockIdx.y;
  const double ai = a[i];
  if (ai == 0.0) return;
  const double* x = (const double*)X.col[i];
  double* y = (double*)Y.col[i];
  const double* x2 = (const double*)X2.col[i];
  double* y2 = (double*)Y2.col[i];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    y[r] += s * ai * x[r];
    if (two) y2[r] += s2 * ai * x2[r];
  }
}

// P_i = Z_i + b_i P_i
__global__ void adj_xpby_cols_kernel(long n, blk_cols Z, blk_cols P, const double* b)
{
  const int i = blockIdx.y;
  const double bi = b[i];
  const double* z = (const double*)Z.col[i];
  double* p = (double*)P.col[i];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    p[r] = z[r] + bi * p[r];
}

// Q_i -= lam_i T_i
__global__ void adj_shift_cols_kernel(long n, blk_cols T, blk_cols Q, const double* lam)
{
  const int i = blockIdx.y;
  const double li = lam[i];
  const double* t = (const double*)T.col[i];
  double* q = (double*)Q.col[i];
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x)
    q[r] -= li * t[r];
}

namespace {

struct adj_state {
  gpu_Context* ctx;
  long n;
  int k;
  gpu_MultiVector *X, *BX, *G, *W;
  gpu_MultiVector *mu, *r, *z, *p, *q, *t, *zo;
  double *Sg, *M, *lam, *glam, *num, *den, *alpha, *rho, *rho2, *bn2;
};

unsigned row_blocks(gpu_Context* ctx, long n, int w)
{
  long want = (n + 255) / 256, cap = (long)ctx->num_sms * 8 / (w > 0 ? w : 1);
  if (cap < 4) cap = 4;
  if (want > cap) want = cap;
  return (unsigned)(want < 1 ? 1 : want);
}

int cols_of(gpu_MultiVector* x, blk_cols* c) { return gb_mv_fill_cols(x, c, 0); }

int apply(adj_state* a, op_fn op, void* data, gpu_MultiVector* x, gpu_MultiVector* y)
{
  gpu_Context* ctx = a->ctx;
  if (op == gpu_OperatorApply) {
    ctx->err[0] = 0;
    op(data, x, y);
    return ctx->err[0] ? -1 : 0;
  }
  if (gb_sync(ctx)) return -1;
  op(data, x, y);
  return gb_cuda_check(ctx, (int)cudaDeviceSynchronize(), "adjoint operator callback");
}

// y <- y - L (R' y) with (L, R) = (BX, X) for P_L and (X, BX) for P_R
int project(adj_state* a, gpu_MultiVector* L, gpu_MultiVector* R, gpu_MultiVector* y)
{
  blk_cols cl, cr, cy;
  cols_of(L, &cl);
  cols_of(R, &cr);
  cols_of(y, &cy);
  const int k = a->k;
  if (gb_gram(a->ctx, GPU_MV_FLOAT64, a->n, &cr, k, &cy, k, a->M, k)) return -1;
  adj_neg_kernel<<<(k * k + 255) / 256, 256, 0, S(a->ctx)>>>(k * k, a->M);
  gb_count_launch(1);
  return gb_bymat(a->ctx, GPU_MV_FLOAT64, a->n, &cl, k, a->M, k, &cy, k, &cy);
}

int dots(adj_state* a, gpu_MultiVector* x, gpu_MultiVector* y, double* out)
{
  blk_cols cx, cy;
  cols_of(x, &cx);
  cols_of(y, &cy);
  int idx[BLK_MAXCOLS];
  for (int i = 0; i < a->k; i++) idx[i] = i;
  return gb_dot_cols(a->ctx, GPU_MV_FLOAT64, a->n, &cx, &cy, a->k, out, idx);
}

// z = P_R T r
int precond(adj_state* a, op_fn T, void* Tdata)
{
  if (T) {
    if (apply(a, T, Tdata, a->r, a->z)) return -1;
  } else {
    blk_cols cr, cz;
    cols_of(a->r, &cr);
    cols_of(a->z, &cz);
    if (gb_axpby(a->ctx, GPU_MV_FLOAT64, a->n, 1.0, &cr, 0.0, &cz, a->k)) return -1;
  }
  return project(a, a->X, a->BX, a->z);
}

}  // namespace

extern "C" int gpu_EigenvectorAdjoint(gpu_MultiVector* X, const double* lambda, gpu_MultiVector* G,
                                      const double* glam, void* Adata, op_fn A, void* Bdata, op_fn B,
                                      void* Tdata, op_fn T, double tol, int maxit,
                                      gpu_MultiVector* W, double* xg, int* iterations,
                                      double* max_rel_residual)
{
  gpu_Context* ctx = X->ctx;
  adj_state a;
  memset(&a, 0, sizeof(a));
  a.ctx = ctx;
  a.n = X->size;
  a.k = X->num_active;
  a.X = X;
  a.G = G;
  a.W = W;
  const int k = a.k;
  if (iterations) *iterations = 0;
  if (max_rel_residual) *max_rel_residual = 0.0;
  if (k < 1) return gb_fail(ctx, "adjoint: empty block");
  if (X->dtype != GPU_MV_FLOAT64 || W->dtype != GPU_MV_FLOAT64 || (G && G->dtype != GPU_MV_FLOAT64))
    return gb_fail(ctx, "adjoint: FP64 blocks expected");
  if (W->num_active != k || (G && G->num_active != k) || W->size != a.n || (G && G->size != a.n))
    return gb_fail(ctx, "adjoint: block sizes differ");
  if (!A) return gb_fail(ctx, "adjoint: operator A missing");

  const size_t kk = (size_t)k * k;
  double* small = (double*)gb_device_alloc(ctx, sizeof(double) * (2 * kk + 10 * (size_t)k) + 64);
  if (!small) return -1;
  a.Sg = small;
  a.M = a.Sg + kk;
  a.lam = a.M + kk;
  a.glam = a.lam + k;
  a.num = a.glam + k;
  a.den = a.num + k;
  a.alpha = a.den + k;
  a.rho = a.alpha + k;
  a.rho2 = a.rho + k;
  a.bn2 = a.rho2 + k;
  gpu_MultiVector* blocks[7] = {NULL, NULL, NULL, NULL, NULL, NULL, NULL};
  int rc = 0, it = 0;
  double worst = 0.0;
  double* host = (double*)malloc(sizeof(double) * 2 * k);
  if (!host) rc = gb_fail(ctx, "adjoint: host allocation failed");
  if (!rc) rc = gb_memcpy_h2d(ctx, a.lam, lambda, sizeof(double) * k);
  if (!rc) {
    if (glam)
      rc = gb_memcpy_h2d(ctx, a.glam, glam, sizeof(double) * k);
    else
      rc = cudaMemsetAsync(a.glam, 0, sizeof(double) * k, S(ctx)) == cudaSuccess ? 0 : -1;
  }
  for (int b = 0; b < 7 && !rc; b++) {
    blocks[b] = gb_mv_create_like(X, GPU_MV_FLOAT64);
    if (!blocks[b]) rc = -1;
  }
  if (!rc) {
    a.mu = blocks[0];
    a.r = blocks[1];
    a.z = blocks[2];
    a.p = blocks[3];
    a.q = blocks[4];
    a.t = blocks[5];
    a.zo = blocks[6];
    gpu_MultiVector* all[7] = {a.mu, a.r, a.z, a.p, a.q, a.t, a.zo};
    for (int b = 0; b < 7; b++) gb_mv_set_mask_host(all[b], NULL);
  }
  // B X (X itself when B is the identity)
  gpu_MultiVector* BXb = NULL;
  if (!rc && B) {
    BXb = gb_mv_create_like(X, GPU_MV_FLOAT64);
    if (!BXb || apply(&a, B, Bdata, X, BXb)) rc = -1;
  }
  a.BX = BXb ? BXb : X;

  blk_cols cx, cbx, cg, cw, cmu, cr, cz, cp, cq, ct, czo;
  if (!rc) {
    cols_of(X, &cx);
    cols_of(a.BX, &cbx);
    cols_of(W, &cw);
    cols_of(a.mu, &cmu);
    cols_of(a.r, &cr);
    cols_of(a.z, &cz);
    cols_of(a.p, &cp);
    cols_of(a.q, &cq);
    cols_of(a.t, &ct);
    cols_of(a.zo, &czo);
    if (G) cols_of(G, &cg);
  }
  const dim3 cgrid(row_blocks(ctx, a.n, k), k);
  if (!rc && !G) {
    // eigenvalue terms only: W = X diag(glam)
    double lmax = 0.0;
    for (int i = 0; i < k; i++) lmax = fmax(lmax, fabs(lambda[i]));
    adj_inspace_kernel<<<(unsigned)((kk + 255) / 256), 256, 0, S(ctx)>>>(k, a.M, a.lam, a.glam, HUGE_VAL,
                                                                         a.M);
    gb_count_launch(1);
    rc = gb_bymat(ctx, GPU_MV_FLOAT64, a.n, &cx, k, a.M, k, &cw, k, NULL);
    if (xg)
      for (int i = 0; i < k; i++) xg[i] = 0.0;
  } else if (!rc) {
    double lmax = 0.0;
    for (int i = 0; i < k; i++) lmax = fmax(lmax, fabs(lambda[i]));
    const double tol_deg = 1e-12 * (lmax > 0.0 ? lmax : 1.0);
    // S = X'G; x_i'g_i for the mass term; W = X M (in-space part + glam)
    rc = gb_gram(ctx, GPU_MV_FLOAT64, a.n, &cx, k, &cg, k, a.Sg, k);
    if (!rc) {
      adj_inspace_kernel<<<(unsigned)((kk + 255) / 256), 256, 0, S(ctx)>>>(k, a.Sg, a.lam, a.glam,
                                                                           tol_deg, a.M);
      gb_count_launch(1);
      rc = gb_bymat(ctx, GPU_MV_FLOAT64, a.n, &cx, k, a.M, k, &cw, k, NULL);
    }
    if (!rc && xg) {
      double* hs = (double*)malloc(sizeof(double) * kk);
      rc = hs ? gb_memcpy_d2h(ctx, hs, a.Sg, sizeof(double) * kk) : -1;
      if (!rc)
        for (int i = 0; i < k; i++) xg[i] = hs[i + (size_t)i * k];
      free(hs);
    }
    // r = -(I - B X X') G = BX S - G ; mu = 0
    if (!rc) rc = gb_bymat(ctx, GPU_MV_FLOAT64, a.n, &cbx, k, a.Sg, k, &cr, k, NULL);
    if (!rc) rc = gb_axpby(ctx, GPU_MV_FLOAT64, a.n, -1.0, &cg, 1.0, &cr, k);
    if (!rc) rc = gb_axpby(ctx, GPU_MV_FLOAT64, a.n, 0.0, &cr, 0.0, &cmu, k);
    if (!rc) rc = dots(&a, a.r, a.r, a.bn2);
    if (!rc) rc = gb_memcpy_d2h(ctx, host + k, a.bn2, sizeof(double) * k);
    if (!rc) rc = precond(&a, T, Tdata);
    if (!rc) rc = gb_axpby(ctx, GPU_MV_FLOAT64, a.n, 1.0, &cz, 0.0, &cp, k);
    if (!rc) rc = dots(&a, a.r, a.z, a.rho);
    const double tol2 = tol * tol;
    for (it = 1; !rc && it <= maxit; it++) {
      // q = P_L (A - Lambda B) p
      if (apply(&a, A, Adata, a.p, a.q)) {
        rc = -1;
        break;
      }
      if (B) {
        if (apply(&a, B, Bdata, a.p, a.t)) {
          rc = -1;
          break;
        }
        adj_shift_cols_kernel<<<cgrid, 256, 0, S(ctx)>>>(a.n, ct, cq, a.lam);
      } else {
        adj_shift_cols_kernel<<<cgrid, 256, 0, S(ctx)>>>(a.n, cp, cq, a.lam);
      }
      gb_count_launch(1);
      if (project(&a, a.BX, a.X, a.q) || dots(&a, a.p, a.q, a.den)) {
        rc = -1;
        break;
      }
      adj_ratio_kernel<<<1, 256, 0, S(ctx)>>>(k, a.rho, a.den, a.alpha);
      adj_axpy_cols_kernel<<<cgrid, 256, 0, S(ctx)>>>(a.n, cp, cmu, a.alpha, 1.0, cq, cr, -1.0, 1);
      gb_count_launch(2);
      // convergence: |r_i| <= tol |b_i| for every column
      if (dots(&a, a.r, a.r, a.num) || gb_memcpy_d2h(ctx, host, a.num, sizeof(double) * k)) {
        rc = -1;
        break;
      }
      worst = 0.0;
      for (int i = 0; i < k; i++) {
        const double rel = host[k + i] > 0.0 ? host[i] / host[k + i] : 0.0;
        if (rel > worst) worst = rel;
      }
      if (worst <= tol2) break;
      // z_old = z; z = P_R T r; rho2 = r'z - r'z_old (Polak-Ribiere)
      if (gb_axpby(ctx, GPU_MV_FLOAT64, a.n, 1.0, &cz, 0.0, &czo, k) || precond(&a, T, Tdata) ||
          dots(&a, a.r, a.z, a.rho2) || dots(&a, a.r, a.zo, a.num)) {
        rc = -1;
        break;
      }
      adj_sub_kernel<<<1, 256, 0, S(ctx)>>>(k, a.rho2, a.num, a.den);  // den <- r'z - r'z_old
      gb_count_launch(1);
      adj_ratio_kernel<<<1, 256, 0, S(ctx)>>>(k, a.den, a.rho, a.alpha);  // beta
      adj_xpby_cols_kernel<<<cgrid, 256, 0, S(ctx)>>>(a.n, cz, cp, a.alpha);
      gb_count_launch(2);
      double* tswap = a.rho;
      a.rho = a.rho2;
      a.rho2 = tswap;
    }
    if (it > maxit) it = maxit;
    // W += mu
    if (!rc) rc = gb_axpby(ctx, GPU_MV_FLOAT64, a.n, 1.0, &cmu, 1.0, &cw, k);
  }
  if (!rc) rc = gb_cuda_check(ctx, (int)cudaGetLastError(), "adjoint");
  gb_sync(ctx);
  if (iterations) *iterations = G ? it : 0;
  if (max_rel_residual) *max_rel_residual = sqrt(worst);
  for (int b = 0; b < 7; b++) gpu_MultiVectorDestroy(blocks[b]);
  gpu_MultiVectorDestroy(BXb);
  gb_device_free(small);
  free(host);
  fflush(stdout);
  return rc;
}
