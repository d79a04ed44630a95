/*
 * lobpcg_driver.c -- the host side of the GB300 LOBPCG solver (C).
 *
 * lobpcg_solve_double() keeps the reference's signature and semantics
 * (blopex_abstract/krylov/lobpcg.c:332-413 and 502-1388) and runs the
 * iteration on the device:
 *   - the block vectors are gpu_MultiVector objects (column-major, device);
 *   - Gram products, X*C updates, residuals and norms are device kernels;
 *   - the 3k x 3k Gram matrices gramA/gramB, the Cholesky-QR factors and the
 *     Rayleigh-Ritz eigenproblem stay in device memory (FP64);
 *   - per iteration only the eigenvalues, residual norms and factorisation
 *     status words come back to the host (for the soft-locking test, the
 *     histories and the caller's arrays).
 *
 * One iteration performs the same operations, on the same gramA/gramB
 * layout, as the reference loop (lobpcg.c:965-1318): implicit identities
 * XAX = diag(lambda), XBX = RBR = PBP = I, lower blocks computed, Cholesky-QR
 * of R and P with the sizeP = 0 restart when P's factorisation fails, and
 * the same coordinate blocks of the Ritz vectors.
 *
 * Precision (lobpcg_gpu_options.precision):
 *   FP64  -- every block in FP64 (the reference's arithmetic);
 *   MIXED -- the iteration first runs on FP32 copies of the blocks (Gram
 *            sums accumulated in FP64, small matrices in FP64) until the
 *            largest residual drops below opt.fp64_below or stops improving;
 *            the block is then promoted to FP64, re-orthonormalised and
 *            Rayleigh-Ritz'ed in FP64 (the FP64 residual check), and the
 *            iteration continues in FP64 until the tolerance is met.
 */
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

mv_InterfaceInterpreter* gb_mv_interpreter(mv_MultiVectorPtr x);

typedef void (*op_fn)(void*, void*, void*);

typedef struct {
  gpu_Context* ctx;
  long n;
  int k, ny, k3;
  int dt; /* dtype of the current phase */
  int noB, noT, noY;
  void *Adata, *Bdata, *Tdata;
  op_fn A, B, T;
  gpu_MultiVector *X, *R, *P, *W, *AX, *AR, *AP, *BX, *BR, *BP, *Y, *BY;
  /* device small matrices */
  double *gA, *gB, *lamAB, *lam, *norm2, *gYBY, *gYBX, *tYBX;
  int* info;
  /* host */
  double* h_lam;
  double* h_norm;
  int* mask;
  int verbosity;
  lobpcg_Tolerance tol;
} solver_t;

static void err_message(int verbosity, const char* msg)
{
  if (verbosity) {
    fprintf(stderr, "Error in LOBPCG:\n");
    fputs(msg, stderr);
  }
}

static void dump_lambda(const double* norms, const double* lam, int it, int k)
{
  printf("\n");
  printf("Eigenvalue lambda       Residual              \n");
  for (int i = 0; i < k; i++) printf("%22.14e  %22.14e\n", lam[i], fabs(norms[i]));
  printf("\n%d iterations\n", it);
}

static double max_value(const double* v, int k)
{
  double m = v[0];
  for (int i = 1; i < k; i++)
    if (v[i] > m) m = v[i];
  return m;
}

/* ----------------------------------------------------------- block ops */

static void cols(const gpu_MultiVector* x, blk_cols* t) { gb_mv_fill_cols(x, t, 0); }

static int d_copy(solver_t* s, gpu_MultiVector* x, gpu_MultiVector* y)
{
  blk_cols a, b;
  if (x->num_active != y->num_active) return gb_fail(s->ctx, "copy: width mismatch");
  cols(x, &a);
  cols(y, &b);
  return gb_convert(s->ctx, s->n, x->dtype, &a, y->dtype, &b, x->num_active);
}

static int d_axpy(solver_t* s, double alpha, gpu_MultiVector* x, gpu_MultiVector* y)
{
  blk_cols a, b;
  if (x->num_active != y->num_active) return gb_fail(s->ctx, "axpy: width mismatch");
  cols(x, &a);
  cols(y, &b);
  return gb_axpby(s->ctx, x->dtype, s->n, alpha, &a, 1.0, &b, x->num_active);
}

/* G(0:h, 0:w) = x(active)' y(active), leading dimension ldg */
static int d_gram(solver_t* s, gpu_MultiVector* x, gpu_MultiVector* y, double* G, int ldg)
{
  blk_cols a, b;
  cols(x, &a);
  cols(y, &b);
  return gb_gram(s->ctx, x->dtype, s->n, &a, x->num_active, &b, y->num_active, G, ldg);
}

/* y(active, w = y->num_active) = x(active, h = x->num_active) * C */
static int d_bymat(solver_t* s, gpu_MultiVector* x, const double* C, int ldc, gpu_MultiVector* y)
{
  blk_cols a, b;
  cols(x, &a);
  cols(y, &b);
  return gb_bymat(s->ctx, x->dtype, s->n, &a, x->num_active, C, ldc, &b, y->num_active, NULL);
}

/* the same with C upper triangular (a Cholesky-QR factor from gb_cholqr_factor,
   zeros below the diagonal) */
static int d_bymat_tri(solver_t* s, gpu_MultiVector* x, const double* C, int ldc,
                       gpu_MultiVector* y)
{
  blk_cols a, b;
  cols(x, &a);
  cols(y, &b);
  return gb_bymat_tri(s->ctx, x->dtype, s->n, &a, x->num_active, C, ldc, &b, y->num_active);
}

/* apply an operator callback to the active columns of x -> y */
static int d_apply(solver_t* s, op_fn op, void* data, gpu_MultiVector* x, gpu_MultiVector* y)
{
  gpu_Context* ctx = s->ctx;
  if (op == gpu_OperatorApply) {
    ctx->err[0] = 0;
    op(data, x, y);
    return ctx->err[0] ? -1 : 0;
  }
  /* a caller-supplied callback may launch on any stream: order it with the
     solver's stream on both sides */
  if (gb_mv_sync_mask(x) || gb_mv_sync_mask(y) || gb_sync(ctx)) return -1;
  op(data, x, y);
  return gb_cuda_check(ctx, (int)cudaDeviceSynchronize(), "operator callback");
}

/* norms of the residual columns listed by mask (all when mask == NULL):
   host h_norm[i] = sqrt(|r_i' r_i|) (lobpcg.c:237-260) */
static int d_resnorms(solver_t* s, gpu_MultiVector* r, const int* mask)
{
  int idx[BLK_MAXCOLS], na = 0;
  blk_cols a;
  for (int i = 0; i < s->k; i++)
    if (!mask || mask[i]) idx[na++] = i;
  if (na != r->num_active) return gb_fail(s->ctx, "residual norms: mask mismatch");
  cols(r, &a);
  if (gb_dot_cols(s->ctx, r->dtype, s->n, &a, &a, na, s->norm2, idx)) return -1;
  double* tmp = (double*)gb_pinned(s->ctx, sizeof(double) * s->k);
  if (!tmp || gb_memcpy_d2h(s->ctx, tmp, s->norm2, sizeof(double) * s->k)) return -1;
  for (int c = 0; c < na; c++) s->h_norm[idx[c]] = sqrt(fabs(tmp[idx[c]]));
  return 0;
}

/* r(active) = bx(active) * diag(lambda(mask)) (lobpcg.c:1277-1279) */
static int d_bydiag_lambda(solver_t* s, gpu_MultiVector* bx, const int* mask, gpu_MultiVector* r)
{
  int idx[BLK_MAXCOLS], na = 0;
  blk_cols a, b;
  for (int i = 0; i < s->k; i++)
    if (!mask || mask[i]) idx[na++] = i;
  if (na != bx->num_active || na != r->num_active)
    return gb_fail(s->ctx, "bydiag: mask mismatch");
  cols(bx, &a);
  cols(r, &b);
  return gb_scale_cols(s->ctx, bx->dtype, s->n, &a, s->lam, idx, &b, na);
}

static int read_info(solver_t* s, int* info)
{
  int* tmp = (int*)gb_pinned(s->ctx, sizeof(int));
  if (!tmp || gb_memcpy_d2h(s->ctx, tmp, s->info, sizeof(int))) return -1;
  *info = *tmp;
  return 0;
}

/* B-orthonormalise x given bx = B x, r = the Gram block (lobpcg.c:197-232).
   *info: 0 or the Cholesky failure order.  Returns -1 on a CUDA error. */
static int d_implicit_qr(solver_t* s, gpu_MultiVector* x, gpu_MultiVector* bx, double* r, int ld,
                         gpu_MultiVector* z, int* info)
{
  const int m = x->num_active;
  if (d_gram(s, x, bx, r, ld)) return -1;
  if (gb_cholqr_factor(s->ctx, r, ld, m, s->info)) return -1;
  if (read_info(s, info)) return -1;
  if (*info) return 0;
  if (d_copy(s, x, z)) return -1;
  return d_bymat_tri(s, z, r, ld, x);
}

static int d_sygv(solver_t* s, int m, double* w, int* info)
{
  if (gb_sygv(s->ctx, s->gA, s->gB, s->k3, m, s->k, w, s->info, 0.0)) return -1;
  return read_info(s, info);
}

static int fetch_lambda(solver_t* s)
{
  double* tmp = (double*)gb_pinned(s->ctx, sizeof(double) * s->k);
  if (!tmp || gb_memcpy_d2h(s->ctx, tmp, s->lam, sizeof(double) * s->k)) return -1;
  memcpy(s->h_lam, tmp, sizeof(double) * s->k);
  return 0;
}

/* -------------------------------------------------------- allocation */

static void free_blocks(solver_t* s)
{
  gpu_MultiVector** b[] = {&s->R, &s->P, &s->W, &s->AX, &s->AR, &s->AP};
  for (size_t i = 0; i < sizeof(b) / sizeof(b[0]); i++) {
    gpu_MultiVectorDestroy(*b[i]);
    *b[i] = NULL;
  }
  if (!s->noB) {
    gpu_MultiVectorDestroy(s->BX);
    gpu_MultiVectorDestroy(s->BR);
    gpu_MultiVectorDestroy(s->BP);
    if (!s->noY) gpu_MultiVectorDestroy(s->BY);
  }
  s->BX = s->BR = s->BP = s->BY = NULL;
}

static int alloc_blocks(solver_t* s, gpu_MultiVector* X)
{
  gpu_Context* ctx = s->ctx;
  s->X = X;
  s->dt = X->dtype;
  s->R = gb_mv_create_like(X, s->dt);
  s->P = gb_mv_create_like(X, s->dt);
  s->W = gb_mv_create_like(X, s->dt);
  s->AX = gb_mv_create_like(X, s->dt);
  s->AR = gb_mv_create_like(X, s->dt);
  s->AP = gb_mv_create_like(X, s->dt);
  if (!s->R || !s->P || !s->W || !s->AX || !s->AR || !s->AP) return gb_fail(ctx, "out of device memory");
  if (!s->noB) {
    s->BX = gb_mv_create_like(X, s->dt);
    s->BR = gb_mv_create_like(X, s->dt);
    s->BP = gb_mv_create_like(X, s->dt);
    if (!s->BX || !s->BR || !s->BP) return gb_fail(ctx, "out of device memory");
  } else {
    s->BX = s->X;
    s->BR = s->R;
    s->BP = s->P;
  }
  return 0;
}

/* ---------------------------------------------------------- constraints */

/* BY, YBY = chol(BY'Y)^-1 (lobpcg.c:700-751).  Returns 1 on dependent Y. */
static int setup_constraints(solver_t* s, gpu_MultiVector* Yuser)
{
  gpu_Context* ctx = s->ctx;
  int info = 0;
  const int ny = s->ny;
  /* constraints live in the phase dtype */
  if (Yuser->dtype == s->dt) {
    s->Y = Yuser;
  } else {
    s->Y = gb_mv_create_like(Yuser, s->dt);
    if (!s->Y || d_copy(s, Yuser, s->Y)) return -1;
  }
  s->BY = s->Y;
  if (!s->noB) {
    s->BY = gb_mv_create_like(s->Y, s->dt);
    if (!s->BY || d_apply(s, s->B, s->Bdata, s->Y, s->BY)) return -1;
  }
  if (d_gram(s, s->BY, s->Y, s->gYBY, ny)) return -1;
  if (gb_cholqr_factor(ctx, s->gYBY, ny, ny, s->info) || read_info(s, &info)) return -1;
  return info ? 1 : 0;
}

/* x <- x - Y (YBY^-T YBY^-1 (BY' x)) for the active columns of x; W must
   carry the same mask as x (lobpcg.c:742-750, 996-1012) */
static int project_constraints(solver_t* s, gpu_MultiVector* x)
{
  const int ny = s->ny, w = x->num_active;
  if (s->W->num_active != w) return gb_fail(s->ctx, "constraints: W mask mismatch");
  if (d_gram(s, s->BY, x, s->gYBX, ny)) return -1;
  if (gb_small_gemm(s->ctx, s->gYBY, ny, 1, s->gYBX, ny, 0, s->tYBX, ny, ny, w, ny)) return -1;
  if (gb_small_gemm(s->ctx, s->gYBY, ny, 0, s->tYBX, ny, 0, s->gYBX, ny, ny, w, ny)) return -1;
  if (d_bymat(s, s->Y, s->gYBX, ny, s->W)) return -1;
  return d_axpy(s, -1.0, s->W, x);
}

/* --------------------------------------------------------------- phase */

typedef struct {
  int* iteration;       /* global iteration counter (reference semantics) */
  int maxit;
  int it_base;          /* iterations completed before this phase */
  double* lam_hist;
  int lam_gh;
  double* res_hist;
  int res_gh;
  int stop_fp32;        /* FP32 phase: hand over to FP64 on these criteria */
  double fp64_below;
  int stall_limit;
  int handed_over;      /* out: the FP32 phase stopped for the hand-over */
} phase_ctl;

/* the initial B-orthonormalisation + Rayleigh-Ritz of a phase
   (lobpcg.c:853-962).  Returns the reference exit flag or -2 on CUDA error. */
static int phase_setup(solver_t* s)
{
  const int k = s->k, k3 = s->k3;
  int info = 0;
  for (int i = 0; i < k; i++) s->mask[i] = 1;
  gb_mv_set_mask_host(s->R, s->mask);
  gb_mv_set_mask_host(s->P, s->mask);
  gb_mv_set_mask_host(s->AR, s->mask);
  gb_mv_set_mask_host(s->AP, s->mask);
  gb_mv_set_mask_host(s->AX, NULL);
  gb_mv_set_mask_host(s->X, NULL);
  if (!s->noB) {
    gb_mv_set_mask_host(s->BR, s->mask);
    gb_mv_set_mask_host(s->BP, s->mask);
    gb_mv_set_mask_host(s->BX, NULL);
  }
  gb_mv_set_mask_host(s->W, s->mask);

  if (!s->noB && d_apply(s, s->B, s->Bdata, s->X, s->BX)) return -2;
  if (d_implicit_qr(s, s->X, s->BX, s->gB, k3, s->W, &info)) return -2;
  if (info) {
    err_message(s->verbosity, "Bad initial vectors: orthonormalization failed\n");
    if (s->verbosity) printf("DPOTRF INFO = %d\n", info);
    return info;
  }
  if (!s->noB) {
    if (d_bymat(s, s->BX, s->gB, k3, s->W) || d_copy(s, s->W, s->BX)) return -2;
  }
  if (d_apply(s, s->A, s->Adata, s->X, s->AX)) return -2;
  if (d_gram(s, s->X, s->AX, s->gA, k3) || gb_small_symmetrize(s->ctx, s->gA, k3, k)) return -2;
  if (d_gram(s, s->X, s->BX, s->gB, k3) || gb_small_symmetrize(s->ctx, s->gB, k3, k)) return -2;
  if (d_sygv(s, k, s->lam, &info)) return -2;
  if (info) {
    err_message(s->verbosity, "Bad problem: Rayleigh-Ritz in the initial subspace failed\n");
    if (s->verbosity) printf("DSYGV INFO = %d\n", info);
    return info;
  }
  if (d_bymat(s, s->X, s->gA, k3, s->W) || d_copy(s, s->W, s->X)) return -2;
  if (d_bymat(s, s->AX, s->gA, k3, s->W) || d_copy(s, s->W, s->AX)) return -2;
  if (!s->noB && (d_bymat(s, s->BX, s->gA, k3, s->W) || d_copy(s, s->W, s->BX))) return -2;
  if (d_bydiag_lambda(s, s->BX, NULL, s->R) || d_axpy(s, -1.0, s->AX, s->R)) return -2;
  if (d_resnorms(s, s->R, NULL) || fetch_lambda(s)) return -2;
  return 0;
}

static int nonfinite(const double* v, int k)
{
  for (int i = 0; i < k; i++)
    if (!isfinite(v[i])) return 1;
  return 0;
}

/* the main loop of one phase (lobpcg.c:965-1318).  Returns the exit flag
   (0 or a factorisation INFO) or -2 on a CUDA error; *ctl->iteration
   follows the reference's counter. */
static int phase_loop(solver_t* s, phase_ctl* ctl)
{
  const int k = s->k, k3 = s->k3;
  int exitflag = 0, info = 0;
  int sizeR, sizeP, sizeA, firstR, lastR, firstP;
  int* it = ctl->iteration;
  double best = HUGE_VAL;
  int stall = 0;

  for (*it = ctl->it_base + 1; exitflag == 0 && *it <= ctl->maxit; (*it)++) {
    /* soft locking (lobpcg.c:265-294) */
    sizeR = 0;
    for (int i = 0; i < k; i++) {
      s->mask[i] = s->h_norm[i] > fabs(s->h_lam[i]) * s->tol.relative + s->tol.absolute + DBL_EPSILON;
      sizeR += s->mask[i];
    }
    if (sizeR < 1) break;
    if (ctl->stop_fp32) {
      double mx = 0.0;
      for (int i = 0; i < k; i++)
        if (s->mask[i] && s->h_norm[i] > mx) mx = s->h_norm[i];
      if (mx < ctl->fp64_below) {
        ctl->handed_over = 1;
        break;
      }
      /* stagnation at the FP32 floor: no new minimum (by 0.1 %) of the
         largest active residual for stall_limit iterations */
      if (mx < 0.999 * best) {
        best = mx;
        stall = 0;
      } else if (++stall >= ctl->stall_limit) {
        ctl->handed_over = 1;
        break;
      }
    }
    gb_mv_set_mask_host(s->R, s->mask);
    gb_mv_set_mask_host(s->P, s->mask);
    gb_mv_set_mask_host(s->AR, s->mask);
    gb_mv_set_mask_host(s->AP, s->mask);
    if (!s->noB) {
      gb_mv_set_mask_host(s->BR, s->mask);
      gb_mv_set_mask_host(s->BP, s->mask);
    }
    gb_mv_set_mask_host(s->W, s->mask);

    if (!s->noT) {
      if (d_apply(s, s->T, s->Tdata, s->R, s->W) || d_copy(s, s->W, s->R)) return -2;
    }
    if (!s->noY && project_constraints(s, s->R)) return -2;

    firstR = k;
    lastR = k + sizeR;
    firstP = lastR;
    double* upR = s->gB + firstR + (size_t)firstR * k3;
    if (!s->noB && d_apply(s, s->B, s->Bdata, s->R, s->BR)) return -2;
    if (d_implicit_qr(s, s->R, s->BR, upR, k3, s->W, &info)) return -2;
    exitflag = info;
    if (exitflag && ctl->stop_fp32) {
      /* FP32 storage cannot orthonormalise R any more: X is still the
         previous iteration's block, continue from it in FP64 */
      ctl->handed_over = 1;
      exitflag = 0;
      break;
    }
    if (exitflag) {
      err_message(s->verbosity, "Orthonormalization of residuals failed\n");
      if (s->verbosity) printf("DPOTRF INFO = %d\n", exitflag);
      break;
    }
    if (!s->noB && (d_bymat_tri(s, s->BR, upR, k3, s->W) || d_copy(s, s->W, s->BR))) return -2;
    if (d_apply(s, s->A, s->Adata, s->R, s->AR)) return -2;

    if (*it > ctl->it_base + 1) {
      double* upP = s->gB + firstP + (size_t)firstP * k3;
      sizeP = sizeR;
      if (d_implicit_qr(s, s->P, s->BP, upP, k3, s->W, &info)) return -2;
      exitflag = info;
      if (exitflag) {
        sizeP = 0; /* lobpcg.c:1056-1063 */
      } else {
        if (!s->noB && (d_bymat_tri(s, s->BP, upP, k3, s->W) || d_copy(s, s->W, s->BP))) return -2;
        if (d_bymat_tri(s, s->AP, upP, k3, s->W) || d_copy(s, s->W, s->AP)) return -2;
      }
    } else {
      sizeP = 0;
    }
    sizeA = lastR + sizeP;

    /* Gram blocks, implicit identities (lobpcg.c:1092-1160) */
    if (gb_small_diag(s->ctx, s->gA, k3, k, s->lam)) return -2;
    if (d_gram(s, s->R, s->AX, s->gA + firstR, k3)) return -2;
    if (d_gram(s, s->R, s->AR, s->gA + firstR + (size_t)firstR * k3, k3)) return -2;
    if (gb_small_symmetrize(s->ctx, s->gA + firstR + (size_t)firstR * k3, k3, sizeR)) return -2;
    if (gb_small_identity(s->ctx, s->gB, k3, k, k)) return -2;
    if (d_gram(s, s->R, s->BX, s->gB + firstR, k3)) return -2;
    if (gb_small_identity(s->ctx, upR, k3, sizeR, sizeR)) return -2;
    if (*it > ctl->it_base + 1) {
      double* aP = s->gA + firstP;
      if (d_gram(s, s->P, s->AX, aP, k3)) return -2;
      if (d_gram(s, s->P, s->AR, aP + (size_t)firstR * k3, k3)) return -2;
      if (d_gram(s, s->P, s->AP, aP + (size_t)firstP * k3, k3)) return -2;
      if (gb_small_symmetrize(s->ctx, aP + (size_t)firstP * k3, k3, sizeR)) return -2;
      if (d_gram(s, s->P, s->BX, s->gB + firstP, k3)) return -2;
      if (d_gram(s, s->P, s->BR, s->gB + firstP + (size_t)firstR * k3, k3)) return -2;
      if (gb_small_identity(s->ctx, s->gB + firstP + (size_t)firstP * k3, k3, sizeR, sizeR))
        return -2;
    }

    /* Rayleigh-Ritz (lobpcg.c:1164-1181) */
    if (d_sygv(s, sizeA, s->lamAB, &info)) return -2;
    exitflag = info;
    if (exitflag != 0 && ctl->stop_fp32) {
      ctl->handed_over = 1;
      exitflag = 0;
      break;
    }
    if (exitflag != 0) {
      err_message(s->verbosity, "GEVP solver failure\n");
      fprintf(stderr, "Return Code %d\n", exitflag);
      printf("INFO = %d\n", exitflag);
      fflush(stdout);
      (*it)--;
      break;
    }
    if (gb_memcpy_d2d(s->ctx, s->lam, s->lamAB, sizeof(double) * k)) return -2;

    /* P and X updates (lobpcg.c:1191-1272); coordinates are columns 0..k-1
       of gramA, rows firstR.. for R and firstP.. for P */
    const double* cX = s->gA;
    const double* cR = s->gA + firstR;
    const double* cP = s->gA + firstP;
    if (*it > ctl->it_base + 1) {
      gb_mv_set_mask_host(s->W, NULL);
      if (d_bymat(s, s->P, cP, k3, s->W)) return -2;
      gb_mv_set_mask_host(s->P, NULL);
      if (d_copy(s, s->W, s->P)) return -2;
      if (d_bymat(s, s->AP, cP, k3, s->W)) return -2;
      gb_mv_set_mask_host(s->AP, NULL);
      if (d_copy(s, s->W, s->AP)) return -2;
      if (!s->noB) {
        if (d_bymat(s, s->BP, cP, k3, s->W)) return -2;
        gb_mv_set_mask_host(s->BP, NULL);
        if (d_copy(s, s->W, s->BP)) return -2;
      }
      if (d_bymat(s, s->R, cR, k3, s->W) || d_axpy(s, 1.0, s->W, s->P)) return -2;
      if (d_bymat(s, s->AR, cR, k3, s->W) || d_axpy(s, 1.0, s->W, s->AP)) return -2;
      if (!s->noB && (d_bymat(s, s->BR, cR, k3, s->W) || d_axpy(s, 1.0, s->W, s->BP))) return -2;
    } else {
      gb_mv_set_mask_host(s->P, NULL);
      if (d_bymat(s, s->R, cR, k3, s->P)) return -2;
      gb_mv_set_mask_host(s->AP, NULL);
      if (d_bymat(s, s->AR, cR, k3, s->AP)) return -2;
      if (!s->noB) {
        gb_mv_set_mask_host(s->BP, NULL);
        if (d_bymat(s, s->BR, cR, k3, s->BP)) return -2;
      }
    }
    gb_mv_set_mask_host(s->W, NULL);
    if (d_copy(s, s->X, s->W) || d_bymat(s, s->W, cX, k3, s->X) || d_axpy(s, 1.0, s->P, s->X))
      return -2;
    if (d_copy(s, s->AX, s->W) || d_bymat(s, s->W, cX, k3, s->AX) || d_axpy(s, 1.0, s->AP, s->AX))
      return -2;
    if (!s->noB) {
      if (d_copy(s, s->BX, s->W) || d_bymat(s, s->W, cX, k3, s->BX) ||
          d_axpy(s, 1.0, s->BP, s->BX))
        return -2;
    }

    /* residuals of the active columns (lobpcg.c:1274-1286) */
    gb_mv_set_mask_host(s->AX, s->mask);
    gb_mv_set_mask_host(s->BX, s->mask);
    if (d_bydiag_lambda(s, s->BX, s->mask, s->R) || d_axpy(s, -1.0, s->AX, s->R)) return -2;
    if (d_resnorms(s, s->R, s->mask) || fetch_lambda(s)) return -2;
    if (nonfinite(s->h_lam, k)) {
      gb_fail(s->ctx, "non-finite Ritz values");
      return -2;
    }

    {
      const int col = *it;
      if (ctl->lam_hist && col <= ctl->maxit)
        memcpy(ctl->lam_hist + (size_t)col * ctl->lam_gh, s->h_lam, sizeof(double) * k);
      if (ctl->res_hist && col <= ctl->maxit)
        memcpy(ctl->res_hist + (size_t)col * ctl->res_gh, s->h_norm, sizeof(double) * k);
    }
    if (s->verbosity == 2) {
      printf("Iteration %d \tbsize %d\n", *it, sizeR);
      dump_lambda(s->h_norm, s->h_lam, *it, k);
    } else if (s->verbosity == 1) {
      printf("Iteration %d \tbsize %d \tmaxres %22.14e\n", *it, sizeR, max_value(s->h_norm, k));
    }

    gb_mv_set_mask_host(s->AX, NULL);
    gb_mv_set_mask_host(s->BX, NULL);
    gb_mv_set_mask_host(s->AP, s->mask);
    gb_mv_set_mask_host(s->BP, s->mask);
    gb_mv_set_mask_host(s->P, s->mask);
    gb_mv_set_mask_host(s->W, s->mask);
  }
  return exitflag;
}

/* ------------------------------------------------- explicit-Gram phase */

/* a step whose largest active residual grows by more than this is undone */
#define EXPLICIT_JUMP 20.0
/* split mode: consecutive undone steps before the hand-over to FP64 */
#define SPLIT_MAX_UNDOS 3

static size_t dt_size(int dtype) { return dtype == GPU_MV_FLOAT64 ? 8 : 4; }

/* column table entries for columns idx[0..n) of x, appended at offset */
static int cols_idx(const gpu_MultiVector* x, const int* idx, int n, blk_cols* t, int off)
{
  const char* base = (const char*)x->data;
  const size_t stride = dt_size(x->dtype) * (size_t)x->ld;
  for (int c = 0; c < n; c++) t->col[off + c] = base + stride * (idx ? idx[c] : c);
  return off + n;
}

static void set_prefix(gpu_MultiVector* x, int n)
{
  x->num_active = n;
  for (int c = 0; c < n; c++) x->active[c] = c;
}

typedef struct {
  gpu_MultiVector *Xn, *AXn, *BXn, *Pn, *APn, *BPn;
  double *G, *H, *Gs, *Hs, *T, *G2, *H2, *tmp, *d, *w;
  int* infos; /* device: 3 Cholesky status words */
  /* FP64 accumulation: X and AX in FP64 (double-buffered), the caller's
     FP64 block that receives X at the end, scratch for Rayleigh quotients */
  gpu_MultiVector *X64[2], *AX64[2], *Xout;
  double* rq;
  int wrote_x64;
  int* pdrop; /* device: P columns dropped by the deflating Cholesky */
  /* split products (FP64-carried X): RS = lambda X - A X for all k columns
     (FP32) and Hx = X'[X R P] (FP64, k x 3k) */
  gpu_MultiVector* RS;
  double* Hx;
} explicit_bufs;

/* exact A X in FP64 every this many FP64-accumulated steps (in between, AX is
   updated by FP32 corrections like X) */
#define ACC64_REFRESH 8

/* Block-orthonormalise the explicit pencil on the small side: with U_b the
   upper Cholesky factor of the b-th diagonal block of H (b = X, R, P),
   T = blockdiag(inv(U_X), inv(U_R), inv(U_P)), G2 = T'GT, H2 = T'HT.  This is
   the reference's Cholesky-QR of R and P (lobpcg.c:197-232, 1027-1077)
   applied to the Gram matrices instead of the n x k blocks.  *bad: bit 1 if
   R's block is not definite, bit 2 for P's. */
static int explicit_orthonormalise(solver_t* s, explicit_bufs* eb, int nR, int nP, int* bad)
{
  const int k = s->k, k3 = s->k3, m = k + nR + nP;
  const int off[3] = {0, k, k + nR}, sz[3] = {k, nR, nP};
  if (gb_small_identity(s->ctx, eb->T, k3, m, m)) return -1;
  for (int b = 0; b < 3; b++) {
    if (sz[b] == 0) continue;
    double* Tb = eb->T + off[b] + (size_t)off[b] * k3;
    /* T_bb <- H_bb, then inv(chol(H_bb)) in place; P's block drops only the
       columns that are not resolved (directions already in span [X R]) */
    if (gb_small_copy(s->ctx, eb->H + off[b] + (size_t)off[b] * k3, k3, Tb, k3, sz[b], sz[b]))
      return -1;
    if (b == 2) {
      if (gb_chol_deflate(s->ctx, Tb, k3, sz[b], s->ctx->opt.explicit_pivot_below, eb->pdrop,
                          eb->infos + 3))
        return -1;
    } else if (gb_cholqr_factor(s->ctx, Tb, k3, sz[b], eb->infos + b)) {
      return -1;
    }
  }
  int* hinfo = (int*)gb_pinned(s->ctx, sizeof(int) * 4);
  if (!hinfo || gb_memcpy_d2h(s->ctx, hinfo, eb->infos, sizeof(int) * 4)) return -1;
  const int ndrop = sz[2] ? hinfo[3] : 0;
  *bad = (sz[0] && hinfo[0] ? 1 : 0) | (sz[1] && hinfo[1] ? 2 : 0) | (sz[2] && ndrop == sz[2] ? 4 : 0);
  if (*bad) return 0;
  s->ctx->stats.explicit_p_drops += ndrop;
  /* G2 = T' G T, H2 = T' H T */
  if (gb_small_gemm(s->ctx, eb->G, k3, 0, eb->T, k3, 0, eb->tmp, k3, m, m, m)) return -1;
  if (gb_small_gemm(s->ctx, eb->T, k3, 1, eb->tmp, k3, 0, eb->G2, k3, m, m, m)) return -1;
  if (gb_small_gemm(s->ctx, eb->H, k3, 0, eb->T, k3, 0, eb->tmp, k3, m, m, m)) return -1;
  if (gb_small_gemm(s->ctx, eb->T, k3, 1, eb->tmp, k3, 0, eb->H2, k3, m, m, m)) return -1;
  if (ndrop && gb_deflate_pencil(s->ctx, eb->G2, eb->H2, k3, m, off[2], sz[2], eb->pdrop, k))
    return -1;
  return 0;
}

/* R(0:nR) = BX(act) diag(lambda(act)) - AX(act), norms of those columns
   (from FP64 BX, AX into the FP32 R when they are FP64) */
static int explicit_residual(solver_t* s, gpu_MultiVector* X, gpu_MultiVector* AX,
                             gpu_MultiVector* BX, const int* act, int nR)
{
  blk_cols bx, ax, r;
  cols_idx(BX, act, nR, &bx, 0);
  cols_idx(AX, act, nR, &ax, 0);
  cols_idx(s->R, NULL, nR, &r, 0);
  (void)X;
  const int dt = (AX->dtype == GPU_MV_FLOAT64 && s->R->dtype == GPU_MV_FLOAT32) ? GB_RESID_64TO32 : s->dt;
  if (gb_residual(s->ctx, dt, s->n, &bx, &ax, s->lam, act, &r, nR, s->norm2)) return -1;
  double* tmp = (double*)gb_pinned(s->ctx, sizeof(double) * s->k);
  if (!tmp || gb_memcpy_d2h(s->ctx, tmp, s->norm2, sizeof(double) * s->k)) return -1;
  for (int c = 0; c < nR; c++) s->h_norm[act[c]] = sqrt(fabs(tmp[act[c]]));
  return 0;
}

/* split products: RS = lambda X64 - AX64 for all k columns (FP32) and, for
   the columns listed in act (all when act == NULL), the FP64 residual norms
   into h_norm */
static int split_residual(solver_t* s, explicit_bufs* eb, gpu_MultiVector* X64,
                          gpu_MultiVector* AX64, const int* act, int nact)
{
  const int k = s->k;
  int all[BLK_MAXCOLS];
  blk_cols x, ax, r;
  for (int i = 0; i < k; i++) all[i] = i;
  cols_idx(X64, NULL, k, &x, 0);
  cols_idx(AX64, NULL, k, &ax, 0);
  cols_idx(eb->RS, NULL, k, &r, 0);
  if (gb_residual(s->ctx, GB_RESID_64TO32, s->n, &x, &ax, s->lam, all, &r, k, s->norm2)) return -1;
  double* tmp = (double*)gb_pinned(s->ctx, sizeof(double) * k);
  if (!tmp || gb_memcpy_d2h(s->ctx, tmp, s->norm2, sizeof(double) * k)) return -1;
  if (!act)
    for (int i = 0; i < k; i++) s->h_norm[i] = sqrt(fabs(tmp[i]));
  else
    for (int c = 0; c < nact; c++) s->h_norm[act[c]] = sqrt(fabs(tmp[act[c]]));
  return 0;
}

/*
 * The explicit phase of the mixed mode: block LOBPCG with explicit Gram
 * matrices.  Each iteration forms the pencil G = [X R P]'[AX AR AP],
 * H = [X R P]'[BX BR BP] (no separate orthonormalisation passes over R and
 * P), orthonormalises it on the small side and solves it in FP64 on the
 * device -- dropping P when its block is not definite (the restart of
 * lobpcg.c:1056-1063 done on the small side) -- and updates
 * P = [R P] C_RP, X = X C_X + P and their images.  Two variants:
 *   split (B = I, no constraints, k <= 64, the tensor-core kernels usable):
 *     X and A X carried in FP64, the pencil from FP64-accurate split-operand
 *     Grams (oz_gram.cu; the X rows in residual form), X and A X updated by
 *     the split-operand block update (oz_xc.cu); iterates to the tolerance;
 *   FP32: FP32 blocks, TF32 / compensated tensor-core or CUDA-core
 *     products; hands over to the FP64 iteration at its floor.
 * Returns 0 (converged, maxit, or handed over to FP64 with
 * ctl->handed_over set) or -2 on a CUDA error.
 */
static int phase_explicit(solver_t* s, phase_ctl* ctl, explicit_bufs* eb)
{
  const int k = s->k, k3 = s->k3;
  int* it = ctl->iteration;
  int act[BLK_MAXCOLS], prev_act[BLK_MAXCOLS];
  int nR = k, prev_nR = k, nP = 0, haveP = 0, prev_haveP = 0;
  double prev_lam[BLK_MAXCOLS], prev_norm[BLK_MAXCOLS];
  double best = HUGE_VAL;
  int stall = 0;
  gpu_MultiVector *X = s->X, *AX = s->AX, *BX = s->noB ? X : s->BX;
  gpu_MultiVector *P = s->P, *AP = s->AP, *BP = s->noB ? P : s->BP;
  gpu_MultiVector *Xn = eb->Xn, *AXn = eb->AXn, *BXn = s->noB ? eb->Xn : eb->BXn;
  gpu_MultiVector *Pn = eb->Pn, *APn = eb->APn, *BPn = s->noB ? eb->Pn : eb->BPn;
  gpu_MultiVector *R = s->R, *AR = s->AR, *BR = s->noB ? s->R : s->BR;
  int rc = 0;
  /* Gram products on the tensor cores (tcgen05, TF32 products; hi+lo
     compensated once the residuals are small or TF32 stalls) when the block
     fits the kernel; else the FP32 CUDA-core kernel */
  int tc_ok = s->ctx->opt.tensor_cores && s->noB && s->dt == GPU_MV_FLOAT32 && k <= 64;
  {
    /* the tensor-core kernel copies 16-byte pieces of every column */
    const gpu_MultiVector* blocks[8] = {X, AX, P, AP, Xn, AXn, Pn, APn};
    for (int b = 0; b < 8; b++)
      if (((uintptr_t)blocks[b]->data & 15) || (blocks[b]->ld & 3)) tc_ok = 0;
    if (((uintptr_t)R->data & 15) || (R->ld & 3) || ((uintptr_t)AR->data & 15) || (AR->ld & 3) ||
        ((uintptr_t)s->W->data & 15) || (s->W->ld & 3))
      tc_ok = 0;
  }
  int comp = 0;
  int split_undos = 0; /* consecutive undone steps in split mode */
  int timed_out = 0;   /* a tensor-core kernel reported a timed-out wait */
  for (int i = 0; i < k; i++) prev_act[i] = i;  /* phase_setup left R for all columns */
  gb_mv_set_mask_host(X, NULL);
  gb_mv_set_mask_host(AX, NULL);
  /* FP64 accumulation (with the tensor-core kernels and B = I): X and AX are
     carried in FP64 and every step adds an FP32 correction computed from the
     FP32 shadows X, AX; residuals and Ritz values (Rayleigh quotients) come
     from the FP64 pair, so the phase is not held at the FP32 rounding floor of
     the blocks.  The Gram products still limit it to ~1e-7 of the spectrum's
     scale, below which the FP64 iteration takes over. */
  const int acc64 = tc_ok && eb->X64[0] && eb->X64[1] && eb->AX64[0] && eb->AX64[1];
  gpu_MultiVector *X64 = eb->X64[0], *X64n = eb->X64[1], *AX64 = eb->AX64[0], *AX64n = eb->AX64[1];
  int refresh = 0;
  gpu_MultiVector* t64;
  /* split products: X and A X carried in FP64 and updated by the FP64-accurate
     split-operand kernel, the X rows of the pencil FP64-accurate (H from the
     split-operand Gram, G in residual form); the FP32 products then only
     shape the corrections, and the phase iterates to the tolerance */
  const int split = acc64 && eb->RS && eb->Hx && s->ctx->opt.split_products && s->noY;
  int rs_stale = 0;
  /* split mode: the FP32 blocks' Grams compensated from the start (TF32
     products alone make P's Gram block indefinite far more often) */
  if (split && s->ctx->opt.compensated_below > 0.0) comp = 1;
  if (acc64) {
    gpu_MultiVector* b4[4] = {X64, X64n, AX64, AX64n};
    for (int b = 0; b < 4; b++) gb_mv_set_mask_host(b4[b], NULL);
    if (d_copy(s, X, X64) || d_apply(s, s->A, s->Adata, X64, AX64)) return -2;
    blk_cols c64, a64;
    cols_idx(X64, NULL, k, &c64, 0);
    cols_idx(AX64, NULL, k, &a64, 0);
    if (gb_rayleigh_quotients(s->ctx, GPU_MV_FLOAT64, s->n, &c64, &a64, k, eb->rq, s->lam) ||
        fetch_lambda(s))
      return -2;
    for (int i = 0; i < k; i++) prev_act[i] = i;
    set_prefix(R, k);
    if (split) {
      gb_mv_set_mask_host(eb->RS, NULL);
      if (split_residual(s, eb, X64, AX64, NULL, k)) return -2;
    } else if (explicit_residual(s, X64, AX64, X64, prev_act, k)) {
      return -2;
    }
  }

  for (*it = ctl->it_base + 1; *it <= ctl->maxit; (*it)++) {
    nR = 0;
    for (int i = 0; i < k; i++) {
      s->mask[i] = s->h_norm[i] > fabs(s->h_lam[i]) * s->tol.relative + s->tol.absolute + DBL_EPSILON;
      if (s->mask[i]) act[nR++] = i;
    }
    if (nR < 1 && split && refresh != 0) {
      /* converged on the updated A X: confirm on the exact one before the
         FP64 phase's check (the updated A X can understate a residual near
         the tolerance by its FP32 terms, and an FP64 iteration costs several
         split ones) */
      refresh = 0;
      gb_mv_set_mask_host(X64, NULL);
      gb_mv_set_mask_host(AX64, NULL);
      if (d_apply(s, s->A, s->Adata, X64, AX64)) return -2;
      blk_cols x0, x1;
      cols_idx(X64, NULL, k, &x0, 0);
      cols_idx(AX64, NULL, k, &x1, 0);
      if (gb_rayleigh_quotients(s->ctx, GPU_MV_FLOAT64, s->n, &x0, &x1, k, eb->rq, s->lam) ||
          fetch_lambda(s) || split_residual(s, eb, X64, AX64, NULL, k))
        return -2;
      rs_stale = 0;
      for (int i = 0; i < k; i++) {
        s->mask[i] = s->h_norm[i] > fabs(s->h_lam[i]) * s->tol.relative + s->tol.absolute + DBL_EPSILON;
        if (s->mask[i]) act[nR++] = i;
      }
    }
    if (nR < 1) break;
    nP = haveP ? nR : 0; /* P restricted to the active columns */
    {
      double mx = 0.0;
      for (int c = 0; c < nR; c++)
        if (s->h_norm[act[c]] > mx) mx = s->h_norm[act[c]];
      if (!split && mx < ctl->fp64_below) {
        ctl->handed_over = 1;
        s->ctx->stats.handover_reason = 1;
        break;
      }
      /* TF32 products carry ~1e-4 relative errors: compensate once the
         residuals approach that fraction of the Ritz values' scale (or the
         absolute threshold, whichever is reached first) */
      double lmax = 0.0;
      for (int i = 0; i < k; i++) lmax = fmax(lmax, fabs(s->h_lam[i]));
      if (tc_ok && !comp && (mx < s->ctx->opt.compensated_below || mx < 1e-3 * lmax)) {
        comp = 1;
        stall = 0;
      }
      /* progress: the mean log residual over all k columns (the largest
         active residual plateaus for long stretches on clustered spectra
         while the others converge); FP32 has reached its floor when that
         mean sets no new minimum (by 0.1 %) for stall_limit iterations */
      double lg = 0.0;
      for (int i = 0; i < k; i++) lg += log(s->h_norm[i] + DBL_MIN);
      lg /= k;
      /* split mode has no FP32 floor to detect: its residuals plateau as
         long as the FP64 loop's do (near the tolerance LOBPCG itself stalls
         for tens of iterations on a 256^3 problem), so only a long stretch
         without progress hands over */
      const int limit = !split ? ctl->stall_limit : 5 * ctl->stall_limit;
      if (lg < best - 1e-3) {
        best = lg;
        stall = 0;
      } else if (++stall >= limit) {
        if (tc_ok && !comp) {
          comp = 1; /* TF32 products stalled: compensate before FP64 */
          stall = 0;
        } else {
          ctl->handed_over = 1;
          s->ctx->stats.handover_reason = 2;
          break;
        }
      }
    }
    /* the residual block must hold exactly the active columns */
    if (split) {
      if (rs_stale) {
        /* an undone step left RS with its residual: that of the kept block */
        if (split_residual(s, eb, X64, AX64, act, 0)) return -2;
        rs_stale = 0;
      }
    } else if (nR != prev_nR || memcmp(act, prev_act, sizeof(int) * nR)) {
      if (acc64 ? explicit_residual(s, X64, AX64, X64, act, nR)
                : explicit_residual(s, X, AX, BX, act, nR))
        return -2;
    }
    set_prefix(R, nR);
    set_prefix(AR, nR);
    set_prefix(s->W, nR);
    if (!s->noB) set_prefix(BR, nR);
    if (split) {
      /* R = T (the active columns of RS) */
      gb_mv_set_mask_host(eb->RS, s->mask);
      if (!s->noT) {
        gpu_MultiVector* t;
        if (d_apply(s, s->T, s->Tdata, eb->RS, s->W)) return -2;
        t = R;
        R = s->W;
        s->W = t;
        s->R = R;
      } else if (d_copy(s, eb->RS, R)) {
        return -2;
      }
      gb_mv_set_mask_host(eb->RS, NULL);
    } else if (!s->noT) {
      gpu_MultiVector* t;
      if (d_apply(s, s->T, s->Tdata, R, s->W)) return -2;
      t = R;
      R = s->W;
      s->W = t;
      if (s->noB) BR = R;
      s->R = R;
    }
    if (!s->noY && project_constraints(s, R)) return -2;
    if (!s->noB && d_apply(s, s->B, s->Bdata, R, BR)) return -2;
    s->ctx->op_accurate = s->ctx->opt.fp32_accurate_op;
    rc = d_apply(s, s->A, s->Adata, R, AR);
    s->ctx->op_accurate = 0;
    if (rc) return -2;

    /* Gram matrices of [X R P(act)] */
    {
      blk_cols left, right;
      int m, off;
      off = cols_idx(X, NULL, k, &left, 0);
      off = cols_idx(R, NULL, nR, &left, off);
      m = cols_idx(P, act, nP, &left, off);
      off = cols_idx(AX, NULL, k, &right, 0);
      off = cols_idx(AR, NULL, nR, &right, off);
      cols_idx(AP, act, nP, &right, off);
      if (split) {
        /* the whole pencil from exact Grams (split-operand tensor-core
           products): X'[X R P], R'[R P AR AP], P'[P AP]; the X rows of G in
           residual form */
        const int F32 = GPU_MV_FLOAT32, F64 = GPU_MV_FLOAT64;
        const size_t sq = (size_t)k3 * k3;
        double *Hx = eb->Hx, *Hr = Hx + sq, *Hp = Hr + sq;
        blk_cols cq[3];
        int qw[3], qdt[3], nq;
        blk_cols cl;
        cols_idx(X64, NULL, k, &cl, 0);
        nq = 0;
        cols_idx(R, NULL, nR, &cq[nq], 0), qw[nq] = nR, qdt[nq++] = F32;
        if (nP) cols_idx(P, act, nP, &cq[nq], 0), qw[nq] = nP, qdt[nq++] = F32;
        if (gb_oz_gram(s->ctx, s->n, &cl, k, F64, nq, cq, qw, qdt, Hx, k)) return -2;
        cols_idx(R, NULL, nR, &cl, 0);
        nq = 0;
        if (nP) cols_idx(P, act, nP, &cq[nq], 0), qw[nq] = nP, qdt[nq++] = F32;
        cols_idx(AR, NULL, nR, &cq[nq], 0), qw[nq] = nR, qdt[nq++] = F32;
        if (nP) cols_idx(AP, act, nP, &cq[nq], 0), qw[nq] = nP, qdt[nq++] = F32;
        if (gb_oz_gram(s->ctx, s->n, &cl, nR, F32, nq, cq, qw, qdt, Hr, nR)) return -2;
        if (nP) {
          cols_idx(P, act, nP, &cl, 0);
          cols_idx(AP, act, nP, &cq[0], 0), qw[0] = nP, qdt[0] = F32;
          if (gb_oz_gram(s->ctx, s->n, &cl, nP, F32, 1, cq, qw, qdt, Hp, nP)) return -2;
        }
        {
          /* RS' [RS X R P] (RS and X's FP32 shadow): the residual-form X rows
             need S' RS; exact for the stored FP32 values like the other
             Grams (the first k columns, RS' RS, are not used) */
          cols_idx(eb->RS, NULL, k, &cl, 0);
          nq = 0;
          cols_idx(X, NULL, k, &cq[nq], 0), qw[nq] = k, qdt[nq++] = F32;
          cols_idx(R, NULL, nR, &cq[nq], 0), qw[nq] = nR, qdt[nq++] = F32;
          if (nP) cols_idx(P, act, nP, &cq[nq], 0), qw[nq] = nP, qdt[nq++] = F32;
          if (gb_oz_gram(s->ctx, s->n, &cl, k, F32, nq, cq, qw, qdt, eb->tmp, k)) return -2;
        }
        if (gb_split_pencil(s->ctx, Hx, Hr, Hp, eb->tmp, eb->G, eb->H, k3, s->lam, k, nR, nP))
          return -2;
        s->ctx->stats.iterations_split++;
      } else if (tc_ok) {
        blk_cols cx, cr, cp, cax, car, cap;
        cols_idx(X, NULL, k, &cx, 0);
        cols_idx(R, NULL, nR, &cr, 0);
        cols_idx(P, act, nP, &cp, 0);
        cols_idx(AX, NULL, k, &cax, 0);
        cols_idx(AR, NULL, nR, &car, 0);
        cols_idx(AP, act, nP, &cap, 0);
        if (gb_tc_gram(s->ctx, s->n, &cx, k, &cr, nR, &cp, nP, &cax, &car, &cap, comp, eb->G,
                       eb->H, k3))
          return -2;
        if (comp) s->ctx->stats.iterations_compensated++;
      } else {
        if (gb_gram(s->ctx, s->dt, s->n, &left, m, &right, m, eb->G, k3)) return -2;
        off = cols_idx(BX, NULL, k, &right, 0);
        off = cols_idx(BR, NULL, nR, &right, off);
        cols_idx(BP, act, nP, &right, off);
        if (gb_gram(s->ctx, s->dt, s->n, &left, m, &right, m, eb->H, k3)) return -2;
      }

      /* Rayleigh-Ritz on the block-orthonormalised pencil; without P when
         P's block or the pencil is not definite (lobpcg.c:1056-1063) */
      int info = 1, bad = 0;
      int use_p = nP;
      if (explicit_orthonormalise(s, eb, nR, nP, &bad)) return -2;
      if (bad & 3) {
        ctl->handed_over = 1;
        s->ctx->stats.handover_reason = 3; /* X or R cannot be orthonormalised in FP32 */
        break;
      }
      if (bad & 4) {
        use_p = 0;
        s->ctx->stats.explicit_p_drops += nP;
        if (explicit_orthonormalise(s, eb, nR, 0, &bad)) return -2;
        if (bad) {
          ctl->handed_over = 1;
          s->ctx->stats.handover_reason = 3;
          break;
        }
      }
      while (1) {
        int mm = k + nR + use_p;
        if (gb_small_copy(s->ctx, eb->G2, k3, eb->Gs, k3, mm, mm) ||
            gb_small_copy(s->ctx, eb->H2, k3, eb->Hs, k3, mm, mm))
          return -2;
        if (gb_sygv(s->ctx, eb->Gs, eb->Hs, k3, mm, k, eb->w, s->info,
                    s->ctx->opt.explicit_pivot_below) ||
            read_info(s, &info))
          return -2;
        if (info == 0 || use_p == 0) break;
        use_p = 0;
        s->ctx->stats.explicit_p_drops++;
        if (explicit_orthonormalise(s, eb, nR, 0, &bad)) return -2;
        if (bad) break;
      }
      if (info != 0 || bad) {
        ctl->handed_over = 1;
        s->ctx->stats.handover_reason = 4;
        break;
      }
      const int mm = k + nR + use_p;
      /* coordinates in the original basis: C = T C' (first k columns) */
      if (gb_small_gemm(s->ctx, eb->T, k3, 0, eb->Gs, k3, 0, eb->tmp, k3, mm, k, mm)) return -2;
      if (gb_small_copy(s->ctx, eb->tmp, k3, eb->Gs, k3, mm, k)) return -2;
      /* keep the previous Ritz values for an undo (eb->d) */
      if (gb_memcpy_d2d(s->ctx, eb->d, s->lam, sizeof(double) * k)) return -2;
      if (gb_memcpy_d2d(s->ctx, s->lam, eb->w, sizeof(double) * k)) return -2;

      /* FP64 accumulation: the FP32 kernels produce the correction
         X (C_X - I) + P, added to the FP64 block below */
      if (acc64 && !split && gb_small_add_diag(s->ctx, eb->Gs, k3, k, -1.0)) return -2;
      /* P = [R P(act)] C_RP ; X = X C_X + P, and the A / B images */
      const double* cX = eb->Gs;
      const double* cRP = eb->Gs + k;
      const int h = nR + use_p;
      gpu_MultiVector* srcs[3][3] = {{R, P, Pn}, {AR, AP, APn}, {BR, BP, BPn}};
      gpu_MultiVector* xs[3][2] = {{X, Xn}, {AX, AXn}, {BX, BXn}};
      const int nsets = s->noB ? 2 : 3;
      for (int q = 0; q < nsets; q++) {
        blk_cols a, y, z, xa;
        int off2 = cols_idx(srcs[q][0], NULL, nR, &a, 0);
        cols_idx(srcs[q][1], act, use_p, &a, off2);
        cols_idx(srcs[q][2], NULL, k, &y, 0);
        cols_idx(xs[q][0], NULL, k, &xa, 0);
        cols_idx(xs[q][1], NULL, k, &z, 0);
        if (split) {
          /* only P and A P here: X and A X follow in FP64 below */
          if (q == 1 && s->ctx->opt.recompute_ap) {
            gb_mv_set_mask_host(Pn, NULL);
            gb_mv_set_mask_host(APn, NULL);
            if (d_apply(s, s->A, s->Adata, Pn, APn)) return -2;
          } else if (gb_tc_xc(s->ctx, s->n, &a, h, cRP, k3, &y, k, NULL)) {
            return -2;
          }
          continue;
        }
        if (q == 1 && s->ctx->opt.recompute_ap) {
          /* A P from P itself: the update [AR AP] C_RP rounds with the
             cancellation between the R and P coefficients (large when R and
             P are nearly dependent), and an A P that drifts from A times P
             corrupts the next pencil in FP32 */
          gb_mv_set_mask_host(Pn, NULL);
          gb_mv_set_mask_host(APn, NULL);
          if (d_apply(s, s->A, s->Adata, Pn, APn)) return -2;
          if (tc_ok ? gb_tc_xc(s->ctx, s->n, &xa, k, cX, k3, &z, k, &y)
                    : gb_bymat(s->ctx, s->dt, s->n, &xa, k, cX, k3, &z, k, &y))
            return -2;
        } else if (tc_ok) {
          if (gb_tc_xc(s->ctx, s->n, &a, h, cRP, k3, &y, k, NULL)) return -2;
          if (gb_tc_xc(s->ctx, s->n, &xa, k, cX, k3, &z, k, &y)) return -2;
        } else {
          if (gb_bymat(s->ctx, s->dt, s->n, &a, h, cRP, k3, &y, k, NULL)) return -2;
          if (gb_bymat(s->ctx, s->dt, s->n, &xa, k, cX, k3, &z, k, &y)) return -2;
        }
      }
      if (split) {
        /* X = X C_X + P and A X = A X C_X + A P with FP64 accuracy (and the
           FP32 shadow of X for the next step's tensor-core Grams) */
        blk_cols x0, x1, z, y32;
        cols_idx(X64, NULL, k, &x0, 0);
        cols_idx(X64n, NULL, k, &x1, 0);
        cols_idx(Pn, NULL, k, &z, 0);
        cols_idx(Xn, NULL, k, &y32, 0);
        if (gb_oz_xc(s->ctx, s->n, &x0, k, cX, k3, &x1, k, &z, GPU_MV_FLOAT32, &y32)) return -2;
        if (++refresh >= ACC64_REFRESH) {
          /* exact A X: the FP32 A P terms drift from A times P */
          refresh = 0;
          if (d_apply(s, s->A, s->Adata, X64n, AX64n)) return -2;
        } else {
          cols_idx(AX64, NULL, k, &x0, 0);
          cols_idx(AX64n, NULL, k, &x1, 0);
          cols_idx(APn, NULL, k, &z, 0);
          if (gb_oz_xc(s->ctx, s->n, &x0, k, cX, k3, &x1, k, &z, GPU_MV_FLOAT32, NULL)) return -2;
        }
        cols_idx(X64n, NULL, k, &x0, 0);
        cols_idx(AX64n, NULL, k, &x1, 0);
        if (gb_rayleigh_quotients(s->ctx, GPU_MV_FLOAT64, s->n, &x0, &x1, k, eb->rq, s->lam))
          return -2;
        t64 = X64; X64 = X64n; X64n = t64;
        t64 = AX64; AX64 = AX64n; AX64n = t64;
      } else if (acc64) {
        blk_cols x0, xd, x1;
        cols_idx(X64, NULL, k, &x0, 0);
        cols_idx(Xn, NULL, k, &xd, 0);
        cols_idx(X64n, NULL, k, &x1, 0);
        if (gb_accumulate64(s->ctx, s->n, &x0, &xd, &x1, k)) return -2;
        cols_idx(AX64, NULL, k, &x0, 0);
        cols_idx(AXn, NULL, k, &xd, 0);
        cols_idx(AX64n, NULL, k, &x1, 0);
        if (++refresh >= ACC64_REFRESH) {
          /* exact A X: the FP32 corrections of AX drift from A X */
          refresh = 0;
          if (d_apply(s, s->A, s->Adata, X64n, AX64n)) return -2;
          if (gb_convert(s->ctx, s->n, GPU_MV_FLOAT64, &x1, GPU_MV_FLOAT32, &xd, k)) return -2;
        } else if (gb_accumulate64(s->ctx, s->n, &x0, &xd, &x1, k)) {
          return -2;
        }
        cols_idx(X64n, NULL, k, &x0, 0);
        if (gb_rayleigh_quotients(s->ctx, GPU_MV_FLOAT64, s->n, &x0, &x1, k, eb->rq, s->lam))
          return -2;
        t64 = X64; X64 = X64n; X64n = t64;
        t64 = AX64; AX64 = AX64n; AX64n = t64;
      }
      /* swap the double buffers */
      gpu_MultiVector* t;
      t = X; X = Xn; Xn = t;
      t = AX; AX = AXn; AXn = t;
      t = P; P = Pn; Pn = t;
      t = AP; AP = APn; APn = t;
      if (!s->noB) {
        t = BX; BX = BXn; BXn = t;
        t = BP; BP = BPn; BPn = t;
      } else {
        BX = X;
        BXn = Xn;
        BP = P;
        BPn = Pn;
      }
      prev_haveP = haveP;
      haveP = 1; /* P holds all k columns from now on */
    }

    /* residuals of the active columns and the new Ritz values */
    memcpy(prev_lam, s->h_lam, sizeof(double) * k);
    memcpy(prev_norm, s->h_norm, sizeof(double) * k);
    if (fetch_lambda(s)) return -2;
    int undo = nonfinite(s->h_lam, k);
    if (tc_ok) {
      int derr = 0;
      if (gb_device_error(s->ctx, &derr)) return -2;
      if (derr) {
        s->ctx->stats.device_errors++;
        /* a tensor-core kernel gave up waiting: its output is incomplete */
        tc_ok = 0;
        undo = 1;
        timed_out = 1;
      }
    }
    if (!undo) {
      if (split ? split_residual(s, eb, X64, AX64, act, nR)
                : acc64 ? explicit_residual(s, X64, AX64, X64, act, nR)
                        : explicit_residual(s, X, AX, BX, act, nR))
        return -2;
      /* A Ritz pair of the FP32 pencil that is not one of the operator
         (Gram errors ~1e-4 with TF32 products) shows as a jump of the
         largest residual: undo the step -- the previous block, its images
         and P are intact in the other buffers -- and continue with more
         precise products (TF32 -> compensated -> FP64). */
      double mo = 0.0, mn = 0.0;
      for (int c = 0; c < nR; c++) {
        mo = fmax(mo, prev_norm[act[c]]);
        mn = fmax(mn, s->h_norm[act[c]]);
      }
      undo = !(mn <= EXPLICIT_JUMP * mo);
    }
    if (undo) {
      gpu_MultiVector* t;
      if (acc64) {
        t = X64; X64 = X64n; X64n = t;
        t = AX64; AX64 = AX64n; AX64n = t;
      }
      t = X; X = Xn; Xn = t;
      t = AX; AX = AXn; AXn = t;
      t = P; P = Pn; Pn = t;
      t = AP; AP = APn; APn = t;
      if (!s->noB) {
        t = BX; BX = BXn; BXn = t;
        t = BP; BP = BPn; BPn = t;
      } else {
        BX = X;
        BXn = Xn;
        BP = P;
        BPn = Pn;
      }
      haveP = prev_haveP;
      memcpy(s->h_lam, prev_lam, sizeof(double) * k);
      memcpy(s->h_norm, prev_norm, sizeof(double) * k);
      if (gb_memcpy_d2d(s->ctx, s->lam, eb->d, sizeof(double) * k)) return -2;
      s->ctx->stats.explicit_undos++;
      if (split && tc_ok && ++split_undos <= SPLIT_MAX_UNDOS) {
        /* with FP64-accurate X rows a jump is LOBPCG's own (the FP64 path
           shows them too): retry the step from the kept block without P,
           the reference's restart (lobpcg.c:1056-1063) taken on purpose */
        comp = 1;
        haveP = 0;
      } else if (!tc_ok || comp) {
        ctl->handed_over = 1;
        s->ctx->stats.handover_reason = timed_out ? 6 : 5;
        break;
      }
      comp = 1;
      stall = 0;
      prev_nR = -1; /* R holds the rejected step's residual: recompute */
      rs_stale = split;
    } else {
      prev_nR = nR;
      memcpy(prev_act, act, sizeof(int) * nR);
      split_undos = 0;
    }
    {
      const int col = *it;
      if (ctl->lam_hist && col <= ctl->maxit)
        memcpy(ctl->lam_hist + (size_t)col * ctl->lam_gh, s->h_lam, sizeof(double) * k);
      if (ctl->res_hist && col <= ctl->maxit)
        memcpy(ctl->res_hist + (size_t)col * ctl->res_gh, s->h_norm, sizeof(double) * k);
    }
    if (s->verbosity == 2) {
      printf("Iteration %d \tbsize %d\n", *it, nR);
      dump_lambda(s->h_norm, s->h_lam, *it, k);
    } else if (s->verbosity == 1) {
      printf("Iteration %d \tbsize %d \tmaxres %22.14e\n", *it, nR, max_value(s->h_norm, k));
    }
  }
  /* a tensor-core kernel that gave up waiting leaves NaN in its output, which
     the checks above may have met first (a block that is not definite, a
     failed Rayleigh-Ritz solve): the error word names the cause */
  if (tc_ok && ctl->handed_over) {
    int derr = 0;
    if (gb_device_error(s->ctx, &derr)) return -2;
    if (derr) {
      s->ctx->stats.device_errors++;
      s->ctx->stats.handover_reason = 6;
    }
  }
  /* the FP64 block goes straight to the caller's block */
  if (acc64 && eb->Xout && !rc) {
    gb_mv_set_mask_host(X64, NULL);
    gb_mv_set_mask_host(eb->Xout, NULL);
    if (d_copy(s, X64, eb->Xout)) return -2;
    eb->wrote_x64 = 1;
  }
  /* the phase's block lives in s->X for the hand-over */
  if (X != s->X) {
    gb_mv_set_mask_host(X, NULL);
    gb_mv_set_mask_host(s->X, NULL);
    rc = d_copy(s, X, s->X);
  }
  s->R = R;
  return rc ? -2 : 0;
}

/* ------------------------------------------------------------ the API */

static int solve_gpu(gpu_MultiVector* Xu, void* Adata, op_fn A, void* Bdata, op_fn B, void* Tdata,
                     op_fn T, gpu_MultiVector* Yu, lobpcg_Tolerance tol, int maxit, int verbosity,
                     int* iterationNumber, double* lambda, double* lamHist, int lamGh,
                     double* resNorms, double* resHist, int resGh)
{
  gpu_Context* ctx = Xu->ctx;
  solver_t s;
  int exitflag = 0;
  double t0 = gb_now();
  long long launches0 = gpu_KernelLaunchCount();

  memset(&s, 0, sizeof(s));
  memset(&ctx->stats, 0, sizeof(ctx->stats));
  cudaMemsetAsync(ctx->dcount, 0, 8 * sizeof(int), (cudaStream_t)ctx->stream);
  ctx->err[0] = 0;
  ctx->potrf_calls = 0;
  ctx->sygv_calls = 0;
  s.ctx = ctx;
  s.n = Xu->size;
  s.k = Xu->num_vectors;
  s.k3 = 3 * s.k;
  s.ny = Yu ? Yu->num_vectors : 0;
  s.noB = B == NULL;
  s.noT = T == NULL;
  s.noY = s.ny == 0;
  s.A = A;
  s.B = B;
  s.T = T;
  s.Adata = Adata;
  s.Bdata = Bdata;
  s.Tdata = Tdata;
  s.tol = tol;
  s.verbosity = verbosity;
  *iterationNumber = 0;

  if (s.k < 1) {
    err_message(verbosity, "The bloc size is wrong.\n");
    return WRONG_BLOCK_SIZE;
  }
  if (s.k > BLK_MAXCOLS / 3) {
    gb_fail(ctx, "block size %d exceeds the supported maximum %d", s.k, BLK_MAXCOLS / 3);
    err_message(verbosity, "The bloc size is wrong.\n");
    return WRONG_BLOCK_SIZE;
  }
  if (Yu && (Yu->size != s.n || s.ny > BLK_MAXCOLS)) {
    gb_fail(ctx, "constraint block has the wrong shape");
    return REQUESTED_ACCURACY_NOT_ACHIEVED;
  }

  /* device small matrices */
  size_t k3sq = (size_t)s.k3 * s.k3;
  size_t small = 2 * k3sq + s.k3 + 3 * (size_t)s.k + 3 * (size_t)(s.ny + 1) * (s.ny + s.k + 1) + 16;
  double* smem = (double*)gb_device_alloc(ctx, sizeof(double) * small);
  s.info = (int*)gb_device_alloc(ctx, sizeof(int) * 4);
  s.h_lam = (double*)calloc(s.k, sizeof(double));
  s.h_norm = (double*)calloc(s.k, sizeof(double));
  s.mask = (int*)calloc(s.k, sizeof(int));
  if (!smem || !s.info || !s.h_lam || !s.h_norm || !s.mask) {
    exitflag = -2;
    goto done;
  }
  cudaMemsetAsync(smem, 0, sizeof(double) * small, (cudaStream_t)ctx->stream);
  s.gA = smem;
  s.gB = s.gA + k3sq;
  s.lamAB = s.gB + k3sq;
  s.lam = s.lamAB + s.k3;
  s.norm2 = s.lam + s.k;
  s.gYBY = s.norm2 + 2 * s.k;
  s.gYBX = s.gYBY + (size_t)(s.ny + 1) * (s.ny + s.k + 1);
  s.tYBX = s.gYBX + (size_t)(s.ny + 1) * (s.ny + s.k + 1);

  {
    const int mixed = ctx->opt.precision == LOBPCG_GPU_MIXED && Xu->dtype == GPU_MV_FLOAT64;
    gpu_MultiVector* X32 = NULL;
    phase_ctl ctl;
    memset(&ctl, 0, sizeof(ctl));
    ctl.iteration = iterationNumber;
    ctl.maxit = maxit;
    ctl.lam_hist = lamHist;
    ctl.lam_gh = lamGh;
    ctl.res_hist = resHist;
    ctl.res_gh = resGh;

    if (verbosity) {
      printf("\nSolving ");
      printf(s.noB ? "standard" : "generalized");
      printf(" eigenvalue problem with");
      if (s.noT) printf("out");
      printf(" preconditioning\n\n");
      printf("block size %d\n\n", s.k);
      if (s.noY)
        printf("No constraints\n\n");
      else if (s.ny > 1)
        printf("%d constraints\n\n", s.ny);
      else
        printf("%d constraint\n\n", s.ny);
    }

    int x64_done = 0; /* the FP32 phase left its FP64-accumulated X in Xu */
    for (int phase = mixed ? 0 : 1; phase < 2; phase++) {
      double tp = gb_now();
      gpu_MultiVector* Xp = Xu;
      if (phase == 0) {
        X32 = gb_mv_create_like(Xu, ctx->opt.explicit_fp64 ? GPU_MV_FLOAT64 : GPU_MV_FLOAT32);
        if (!X32 || d_copy(&s, Xu, X32)) {
          exitflag = -2;
          break;
        }
        Xp = X32;
      } else if (X32 && !x64_done) {
        gb_mv_set_mask_host(X32, NULL);
        gb_mv_set_mask_host(Xu, NULL);
        if (d_copy(&s, X32, Xu)) {
          exitflag = -2;
          break;
        }
      }
      s.dt = Xp->dtype;
      if (alloc_blocks(&s, Xp)) {
        exitflag = -2;
        break;
      }
      if (!s.noY) {
        int rc = setup_constraints(&s, Yu);
        if (rc < 0) {
          exitflag = -2;
          break;
        }
        if (rc > 0) {
          if (verbosity) printf("Cannot handle linear dependent constraints\n");
          exitflag = WRONG_CONSTRAINTS;
          break;
        }
        gb_mv_set_mask_host(s.W, NULL);
        if (project_constraints(&s, s.X)) {
          exitflag = -2;
          break;
        }
      }
      exitflag = phase_setup(&s);
      explicit_bufs eb;
      int have_eb = 0;
      memset(&eb, 0, sizeof(eb));
      if (exitflag == 0 && phase == 0) {
        /* buffers of the explicit-Gram FP32 phase */
        const size_t sq = (size_t)s.k3 * s.k3;
        eb.Xn = gb_mv_create_like(s.X, s.dt);
        eb.AXn = gb_mv_create_like(s.X, s.dt);
        eb.Pn = gb_mv_create_like(s.X, s.dt);
        eb.APn = gb_mv_create_like(s.X, s.dt);
        if (!s.noB) {
          eb.BXn = gb_mv_create_like(s.X, s.dt);
          eb.BPn = gb_mv_create_like(s.X, s.dt);
        }
        eb.G = (double*)gb_device_alloc(ctx, sizeof(double) * (8 * sq + 4 * (size_t)s.k3) + 64 +
                                                 sizeof(int) * (8 + (size_t)s.k3));
        /* FP64 accumulation blocks (used by the tensor-core path, B = I) */
        const int split = ctx->opt.split_products && s.noY && s.dt == GPU_MV_FLOAT32;
        if ((ctx->opt.accum64 || split) && s.noB && ctx->opt.tensor_cores && s.k <= 64) {
          for (int b = 0; b < 2; b++) {
            eb.X64[b] = gb_mv_create_like(s.X, GPU_MV_FLOAT64);
            eb.AX64[b] = gb_mv_create_like(s.X, GPU_MV_FLOAT64);
          }
          eb.Xout = Xu;
          if (split) {
            eb.RS = gb_mv_create_like(s.X, GPU_MV_FLOAT32);
            /* Hx, Hr, Hp: the exact Grams the split pencil is built from */
            eb.Hx = (double*)gb_device_alloc(ctx, sizeof(double) * 3 * (size_t)s.k3 * s.k3);
          }
        }
        have_eb = 1;
        if (!eb.Xn || !eb.AXn || !eb.Pn || !eb.APn || !eb.G || (!s.noB && (!eb.BXn || !eb.BPn))) {
          exitflag = -2;
        } else {
          eb.H = eb.G + sq;
          eb.Gs = eb.H + sq;
          eb.Hs = eb.Gs + sq;
          eb.T = eb.Hs + sq;
          eb.G2 = eb.T + sq;
          eb.H2 = eb.G2 + sq;
          eb.tmp = eb.H2 + sq;
          eb.d = eb.tmp + sq;
          eb.w = eb.d + s.k3;
          eb.rq = eb.w + s.k3;
          eb.infos = (int*)(eb.rq + 2 * (size_t)s.k3);
          eb.pdrop = eb.infos + 8;
        }
      }
      if (exitflag == 0 && (phase == 1 || !mixed)) {
        /* the setup of the (last) FP64 phase: record it as iteration 0 when
           no FP32 iterations ran */
        if (*iterationNumber == 0) {
          if (lamHist) memcpy(lamHist, s.h_lam, sizeof(double) * s.k);
          if (resHist) memcpy(resHist, s.h_norm, sizeof(double) * s.k);
          if (verbosity == 2)
            dump_lambda(s.h_norm, s.h_lam, 0, s.k);
          else if (verbosity == 1)
            printf("\nInitial Max. Residual %22.14e\n", max_value(s.h_norm, s.k));
        }
      } else if (exitflag == 0 && phase == 0) {
        if (lamHist) memcpy(lamHist, s.h_lam, sizeof(double) * s.k);
        if (resHist) memcpy(resHist, s.h_norm, sizeof(double) * s.k);
        if (verbosity == 2)
          dump_lambda(s.h_norm, s.h_lam, 0, s.k);
        else if (verbosity == 1)
          printf("\nInitial Max. Residual %22.14e\n", max_value(s.h_norm, s.k));
      }
      if (exitflag == 0) {
        ctl.it_base = *iterationNumber;
        ctl.stop_fp32 = phase == 0;
        ctl.fp64_below = ctx->opt.fp64_below;
        ctl.stall_limit = ctx->opt.fp32_stall > 0 ? ctx->opt.fp32_stall : 20;
        ctl.handed_over = 0;
        if (phase == 0)
          exitflag = phase_explicit(&s, &ctl, &eb);
        else
          exitflag = phase_loop(&s, &ctl);
        if (phase == 0) {
          /* the loop counter points one past the last finished iteration */
          int done_its = *iterationNumber - 1;
          ctx->stats.iterations_fp32 = done_its;
          ctx->stats.seconds_fp32 = gb_now() - tp;
          if (exitflag == 0) {
            /* hand over to FP64 (also when FP32 met the tolerance: the
               final residual check is done in FP64) */
            *iterationNumber = done_its;
          }
        } else {
          ctx->stats.iterations_fp64 = *iterationNumber - 1 - ctl.it_base;
          ctx->stats.seconds_fp64 = gb_now() - tp;
        }
      }
      if (have_eb) {
        gpu_MultiVectorDestroy(eb.Xn);
        gpu_MultiVectorDestroy(eb.AXn);
        gpu_MultiVectorDestroy(eb.Pn);
        gpu_MultiVectorDestroy(eb.APn);
        gpu_MultiVectorDestroy(eb.BXn);
        gpu_MultiVectorDestroy(eb.BPn);
        for (int b = 0; b < 2; b++) {
          gpu_MultiVectorDestroy(eb.X64[b]);
          gpu_MultiVectorDestroy(eb.AX64[b]);
        }
        gpu_MultiVectorDestroy(eb.RS);
        if (eb.wrote_x64) x64_done = 1;
        gb_sync(ctx);
        gb_device_free(eb.G);
        gb_device_free(eb.Hx);
      }
      if (!s.noY) {
        if (!s.noB && s.BY != s.Y) gpu_MultiVectorDestroy(s.BY);
        if (s.Y != Yu) gpu_MultiVectorDestroy(s.Y);
        s.Y = s.BY = NULL;
      }
      free_blocks(&s);
      if (exitflag != 0) break;
    }
    if (X32) {
      if (exitflag != 0 && exitflag != -2 && *iterationNumber >= 0) {
        /* failure inside the FP32 phase: return its block */
        gb_mv_set_mask_host(X32, NULL);
        gb_mv_set_mask_host(Xu, NULL);
        d_copy(&s, X32, Xu);
      }
      gpu_MultiVectorDestroy(X32);
    }
  }

done:
  if (exitflag == -2) {
    if (verbosity) fprintf(stderr, "Error in LOBPCG:\n%s\n", ctx->err);
    exitflag = REQUESTED_ACCURACY_NOT_ACHIEVED;
  } else if (exitflag == WRONG_CONSTRAINTS) {
    /* returned as is */
  } else if (exitflag != 0 || *iterationNumber > maxit) {
    exitflag = REQUESTED_ACCURACY_NOT_ACHIEVED;
  }
  if (exitflag != WRONG_CONSTRAINTS) (*iterationNumber)--;
  if (*iterationNumber < 0) *iterationNumber = 0;
  if (s.h_lam) memcpy(lambda, s.h_lam, sizeof(double) * s.k);
  if (s.h_norm) memcpy(resNorms, s.h_norm, sizeof(double) * s.k);
  if (verbosity == 1 && exitflag != WRONG_CONSTRAINTS)
    dump_lambda(s.h_norm, s.h_lam, *iterationNumber, s.k);
  gb_sync(ctx);
  gb_device_free(smem);
  gb_device_free(s.info);
  free(s.h_lam);
  free(s.h_norm);
  free(s.mask);
  {
    double mx = 0.0;
    for (int i = 0; i < s.k; i++)
      if (resNorms[i] > mx) mx = resNorms[i];
    ctx->stats.final_max_residual = mx;
  }
  {
    int* c = (int*)gb_pinned(ctx, 8 * sizeof(int));
    if (c && gb_memcpy_d2h(ctx, c, ctx->dcount, 8 * sizeof(int)) == 0) {
      ctx->stats.rr_jacobi32_sweeps = c[0];
      ctx->stats.rr_max_cluster = c[1];
      ctx->stats.rr_fallbacks = c[2];
      ctx->stats.rr_calls = c[3];
      ctx->stats.rr_graded = c[4];
    }
  }
  ctx->stats.seconds_total = gb_now() - t0;
  ctx->stats.kernel_launches = gpu_KernelLaunchCount() - launches0;
  fflush(stdout);
  return exitflag;
}

int lobpcg_solve_double(mv_MultiVectorPtr blockVectorX, void* operatorAData,
                        void (*operatorA)(void*, void*, void*), void* operatorBData,
                        void (*operatorB)(void*, void*, void*), void* operatorTData,
                        void (*operatorT)(void*, void*, void*), mv_MultiVectorPtr blockVectorY,
                        lobpcg_BLASLAPACKFunctions blap_fn, lobpcg_Tolerance tolerance,
                        int maxIterations, int verbosityLevel, int* iterationNumber,
                        double* lambda_values, double* lambdaHistory_values,
                        BlopexInt lambdaHistory_gh, double* residualNorms_values,
                        double* residualNormsHistory_values, BlopexInt residualNormsHistory_gh)
{
  (void)blap_fn;
  *iterationNumber = 0;
  if (!blockVectorX || !gb_is_gpu_interpreter(gb_mv_interpreter(blockVectorX))) {
    if (verbosityLevel)
      fprintf(stderr,
              "Error in LOBPCG:\nthe block vector is not a gpu_MultiVector "
              "(wrap it with the interpreter from GpuSetupInterpreter)\n");
    return REQUESTED_ACCURACY_NOT_ACHIEVED;
  }
  gpu_MultiVector* X = (gpu_MultiVector*)mv_MultiVectorGetData(blockVectorX);
  gpu_MultiVector* Y = NULL;
  if (blockVectorY) {
    if (!gb_is_gpu_interpreter(gb_mv_interpreter(blockVectorY))) {
      if (verbosityLevel) fprintf(stderr, "Error in LOBPCG:\nconstraints are not a gpu_MultiVector\n");
      return REQUESTED_ACCURACY_NOT_ACHIEVED;
    }
    Y = (gpu_MultiVector*)mv_MultiVectorGetData(blockVectorY);
    if (Y->num_vectors == 0) Y = NULL;
  }
  if (cudaSetDevice(X->ctx->device) != cudaSuccess) return REQUESTED_ACCURACY_NOT_ACHIEVED;
  return solve_gpu(X, operatorAData, operatorA, operatorBData, operatorB, operatorTData, operatorT, Y,
                   tolerance, maxIterations, verbosityLevel, iterationNumber, lambda_values,
                   lambdaHistory_values, lambdaHistory_gh, residualNorms_values,
                   residualNormsHistory_values, residualNormsHistory_gh);
}

int lobpcg_solve(mv_MultiVectorPtr blockVectorX, void* operatorAData,
                 void (*operatorA)(void*, void*, void*), void* operatorBData,
                 void (*operatorB)(void*, void*, void*), void* operatorTData,
                 void (*operatorT)(void*, void*, void*), mv_MultiVectorPtr blockVectorY,
                 lobpcg_BLASLAPACKFunctions blap_fn, lobpcg_Tolerance tolerance, int maxIterations,
                 int verbosityLevel, int* iterationNumber, void* lambda_values,
                 void* lambdaHistory_values, BlopexInt lambdaHistory_gh,
                 double* residualNorms_values, double* residualNormsHistory_values,
                 BlopexInt residualNormsHistory_gh, lobpcg_Interpreter* lobpcg,
                 utilities_FortranInterpreter* util)
{
  (void)lobpcg;
  (void)util;
  return lobpcg_solve_double(blockVectorX, operatorAData, operatorA, operatorBData, operatorB,
                             operatorTData, operatorT, blockVectorY, blap_fn, tolerance,
                             maxIterations, verbosityLevel, iterationNumber,
                             (double*)lambda_values, (double*)lambdaHistory_values,
                             lambdaHistory_gh, residualNorms_values, residualNormsHistory_values,
                             residualNormsHistory_gh);
}
