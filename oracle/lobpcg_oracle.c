/*
 * lobpcg_oracle.c -- TEST INFRASTRUCTURE (the oracle), not product code.
 *
 * A CPU restatement, in plain C with scalar loops, of the reference BLOPEX
 * real (double) LOBPCG path:
 *   driver       blopex_abstract/krylov/lobpcg.c:502-1388 (lobpcg_solve)
 *   block ops    blopex_serial_double/multivector/multi_vector.c
 *   small dense  blopex_abstract/utilities/fortran_matrix.c
 * Each function below names the reference lines whose behaviour it restates.
 * The arithmetic order inside the block operations follows the reference's
 * serial loops so that the oracle tracks the reference closely; it is pinned
 * against golden vectors produced by the unmodified reference
 * (the JSON fixtures in tests/golden, made by tests/golden/make_golden.py).
 *
 * It is used only by the tests, by __graft_entry__.smoke() as the checker,
 * and by bench.py as the CPU baseline ("port").  The product never calls it.
 *
 * LAPACK (dsygv, dpotrf) is passed in as function pointers with the
 * Fortran calling convention (scipy.linalg.cython_lapack provides them).
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef void (*dsygv_fn)(int*, char*, char*, int*, double*, int*, double*,
                         int*, double*, double*, int*, int*);
typedef void (*dpotrf_fn)(char*, int*, double*, int*, int*);

/* ------------------------------------------------------------------ */
/* operators                                                           */
/* ------------------------------------------------------------------ */

enum { OP_NONE = 0, OP_CSR = 1, OP_DENSE = 2, OP_DIAG = 3, OP_STENCIL7 = 4,
       OP_STENCIL5 = 5, OP_STENCIL27 = 6, OP_PCG = 7 };

typedef struct {
  int n;
  const int* rowptr;
  const int* colidx;
  const double* vals;
} oracle_csr;

/* 3D 7-point variable-coefficient operator, Dirichlet boundary.
   cx: (nx+1)*ny*nz face coefficients, face (i,j,k) between cells i-1 and i,
   index i + (nx+1)*(j + ny*k); cy: nx*(ny+1)*nz, index i + nx*(j + (ny+1)*k);
   cz: nx*ny*(nz+1), index i + nx*(j + ny*k).  Cell index i + nx*(j + ny*k).
   (A x)_c = sum over the six faces f of c_f * (x_c - x_nbr), x_nbr = 0 outside.
   The optional shift is added to the diagonal. */
typedef struct {
  int nx, ny, nz;
  const double* cx;
  const double* cy;
  const double* cz;
  double shift;
} oracle_st7;

/* 2D 5-point operator on nx*ny cells; cx: (nx+1)*ny, cy: nx*(ny+1). */
typedef struct {
  int nx, ny;
  const double* cx;
  const double* cy;
  double shift;
} oracle_st5;

/* 3D 27-point graph Laplacian plus shift: w holds 13 weights per cell for
   the 13 "forward" neighbour offsets (see st27_offsets); an edge to a
   neighbour outside the grid does not exist.  (A x)_c = shift*x_c +
   sum_{edges (c,d)} w_cd (x_c - x_d). */
typedef struct {
  int nx, ny, nz;
  const double* w;
  double shift;
} oracle_st27;

static const int st27_offsets[13][3] = {
  {1, 0, 0}, {-1, 1, 0}, {0, 1, 0}, {1, 1, 0},
  {-1, -1, 1}, {0, -1, 1}, {1, -1, 1},
  {-1, 0, 1}, {0, 0, 1}, {1, 0, 1},
  {-1, 1, 1}, {0, 1, 1}, {1, 1, 1}};

typedef struct {
  int kind;
  const void* data;
} oracle_op;

/* T ~ inv(A): `iters` steps of conjugate gradients on A y = x from y = 0,
   preconditioned by M (kind OP_NONE: none).  The inner preconditioner of
   HYPRE's LOBPCG driver with -pcgitr (blopex_hypre/krylov/HYPRE_lobpcg.c:
   317-320, a fixed number of PCG steps per application), one column at a
   time; a coefficient with a zero numerator or denominator is 0. */
typedef struct {
  oracle_op A;
  oracle_op M;
  int iters;
} oracle_pcg;

static void op_apply_col(const oracle_op* op, long n, const double* x, double* y);

static void pcg_apply_col(const oracle_pcg* T, long n, const double* x, double* y)
{
  double* w = (double*)calloc(4 * (size_t)n, sizeof(double));
  double *r, *z, *p, *q;
  double rho = 0.0, rho2, pq, alpha, beta;
  long i;
  int it;
  if (!w) {
    for (i = 0; i < n; i++) y[i] = 0.0;
    return;
  }
  r = w;
  z = w + n;
  p = w + 2 * n;
  q = w + 3 * n;
  for (i = 0; i < n; i++) {
    y[i] = 0.0;
    r[i] = x[i];
  }
  if (T->M.kind != OP_NONE)
    op_apply_col(&T->M, n, r, z);
  else
    for (i = 0; i < n; i++) z[i] = r[i];
  for (i = 0; i < n; i++) {
    p[i] = z[i];
    rho += r[i] * z[i];
  }
  for (it = 0; it < T->iters; it++) {
    op_apply_col(&T->A, n, p, q);
    pq = 0.0;
    for (i = 0; i < n; i++) pq += p[i] * q[i];
    alpha = (pq != 0.0 && rho != 0.0) ? rho / pq : 0.0;
    for (i = 0; i < n; i++) {
      y[i] += alpha * p[i];
      r[i] -= alpha * q[i];
    }
    if (it + 1 == T->iters) break;
    if (T->M.kind != OP_NONE)
      op_apply_col(&T->M, n, r, z);
    else
      for (i = 0; i < n; i++) z[i] = r[i];
    rho2 = 0.0;
    for (i = 0; i < n; i++) rho2 += r[i] * z[i];
    beta = (rho != 0.0 && rho2 != 0.0) ? rho2 / rho : 0.0;
    for (i = 0; i < n; i++) p[i] = z[i] + beta * p[i];
    rho = rho2;
  }
  free(w);
}

static void op_apply_col(const oracle_op* op, long n, const double* x, double* y)
{
  long r;
  switch (op->kind) {
  case OP_PCG:
    pcg_apply_col((const oracle_pcg*)op->data, n, x, y);
    break;
  case OP_CSR: {
    const oracle_csr* A = (const oracle_csr*)op->data;
    int p;
    for (r = 0; r < n; r++) {
      double s = 0.0;
      for (p = A->rowptr[r]; p < A->rowptr[r + 1]; p++) s += A->vals[p] * x[A->colidx[p]];
      y[r] = s;
    }
    break;
  }
  case OP_DENSE: {
    /* y = A x with A column-major n*n: restates
       serial_Multi_VectorByMulti_Vector, multi_vector.c:528-576 */
    const double* A = (const double*)op->data;
    long c;
    for (r = 0; r < n; r++) {
      double s = 0.0;
      for (c = 0; c < n; c++) s += A[r + c * n] * x[c];
      y[r] = s;
    }
    break;
  }
  case OP_DIAG: {
    const double* d = (const double*)op->data;
    for (r = 0; r < n; r++) y[r] = d[r] * x[r];
    break;
  }
  case OP_STENCIL7: {
    const oracle_st7* S = (const oracle_st7*)op->data;
    long nx = S->nx, ny = S->ny, nz = S->nz, i, j, k;
    for (k = 0; k < nz; k++)
      for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++) {
          long c = i + nx * (j + ny * k);
          double xc = x[c];
          double cw = S->cx[i + (nx + 1) * (j + ny * k)];
          double ce = S->cx[i + 1 + (nx + 1) * (j + ny * k)];
          double cs = S->cy[i + nx * (j + (ny + 1) * k)];
          double cn = S->cy[i + nx * (j + 1 + (ny + 1) * k)];
          double cb = S->cz[i + nx * (j + ny * k)];
          double ct = S->cz[i + nx * (j + ny * (k + 1))];
          double xw = i > 0 ? x[c - 1] : 0.0;
          double xe = i < nx - 1 ? x[c + 1] : 0.0;
          double xs = j > 0 ? x[c - nx] : 0.0;
          double xn = j < ny - 1 ? x[c + nx] : 0.0;
          double xb = k > 0 ? x[c - nx * ny] : 0.0;
          double xt = k < nz - 1 ? x[c + nx * ny] : 0.0;
          y[c] = (cw + ce + cs + cn + cb + ct + S->shift) * xc
                 - cw * xw - ce * xe - cs * xs - cn * xn - cb * xb - ct * xt;
        }
    break;
  }
  case OP_STENCIL5: {
    const oracle_st5* S = (const oracle_st5*)op->data;
    long nx = S->nx, ny = S->ny, i, j;
    for (j = 0; j < ny; j++)
      for (i = 0; i < nx; i++) {
        long c = i + nx * j;
        double cw = S->cx[i + (nx + 1) * j];
        double ce = S->cx[i + 1 + (nx + 1) * j];
        double cs = S->cy[i + nx * j];
        double cn = S->cy[i + nx * (j + 1)];
        double xw = i > 0 ? x[c - 1] : 0.0;
        double xe = i < nx - 1 ? x[c + 1] : 0.0;
        double xs = j > 0 ? x[c - nx] : 0.0;
        double xn = j < ny - 1 ? x[c + nx] : 0.0;
        y[c] = (cw + ce + cs + cn + S->shift) * x[c] - cw * xw - ce * xe - cs * xs - cn * xn;
      }
    break;
  }
  case OP_STENCIL27: {
    const oracle_st27* S = (const oracle_st27*)op->data;
    long nx = S->nx, ny = S->ny, nz = S->nz, i, j, k;
    int e;
    for (r = 0; r < n; r++) y[r] = S->shift * x[r];
    for (k = 0; k < nz; k++)
      for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++) {
          long c = i + nx * (j + ny * k);
          for (e = 0; e < 13; e++) {
            long i2 = i + st27_offsets[e][0], j2 = j + st27_offsets[e][1],
                 k2 = k + st27_offsets[e][2];
            if (i2 < 0 || i2 >= nx || j2 < 0 || j2 >= ny || k2 < 0 || k2 >= nz) continue;
            {
              long d = i2 + nx * (j2 + ny * k2);
              double w = S->w[13 * c + e];
              double diff = x[c] - x[d];
              y[c] += w * diff;
              y[d] -= w * diff;
            }
          }
        }
    break;
  }
  default:
    break;
  }
}

/* ------------------------------------------------------------------ */
/* block of column vectors with an active-column list                  */
/* (restates serial_Multi_Vector, multi_vector.h:22-32)                */
/* ------------------------------------------------------------------ */

typedef struct {
  double* v;
  long n;
  int k;
  int na;
  int* act;
  int owns;
} blk;

static blk* blk_new(long n, int k, double* storage)
{
  blk* b = (blk*)calloc(1, sizeof(blk));
  int i;
  b->n = n;
  b->k = k;
  b->owns = storage == NULL;
  b->v = storage ? storage : (double*)calloc((size_t)n * (k > 0 ? k : 1), sizeof(double));
  b->act = (int*)malloc(sizeof(int) * (k > 0 ? k : 1));
  for (i = 0; i < k; i++) b->act[i] = i;
  b->na = k;
  return b;
}

static void blk_free(blk* b)
{
  if (!b) return;
  if (b->owns) free(b->v);
  free(b->act);
  free(b);
}

static double* col(const blk* b, int c) { return b->v + (long)b->act[c] * b->n; }

/* multi_vector.c:109-135 */
static void blk_mask(blk* b, const int* mask)
{
  int i;
  b->na = 0;
  for (i = 0; i < b->k; i++)
    if (mask == NULL || mask[i]) b->act[b->na++] = i;
}

/* multi_vector.c:191-222 */
static void blk_copy(const blk* x, blk* y)
{
  int c;
  for (c = 0; c < x->na; c++) memcpy(col(y, c), col(x, c), sizeof(double) * x->n);
}

/* multi_vector.c:251-285 */
static void blk_axpy(double a, const blk* x, blk* y)
{
  int c;
  long r;
  for (c = 0; c < x->na; c++) {
    const double* s = col(x, c);
    double* d = col(y, c);
    for (r = 0; r < x->n; r++) d[r] += a * s[r];
  }
}

/* v(1:h,1:w) = x' y, ld gh: multi_vector.c:354-406 */
static void blk_gram(const blk* x, const blk* y, int gh, double* v)
{
  int i, j;
  long r;
  for (j = 0; j < y->na; j++) {
    const double* yc = col(y, j);
    for (i = 0; i < x->na; i++) {
      const double* xc = col(x, i);
      double s = 0.0;
      for (r = 0; r < x->n; r++) s += xc[r] * yc[r];
      v[i + (long)j * gh] = s;
    }
  }
}

/* y = x * c (c is h x w, ld gh): multi_vector.c:474-524 */
static void blk_bymat(const blk* x, int gh, int h, int w, const double* c, blk* y)
{
  int i, j;
  long r;
  for (j = 0; j < w; j++) {
    double* yc = col(y, j);
    const double* x0 = col(x, 0);
    double a = c[(long)j * gh];
    for (r = 0; r < x->n; r++) yc[r] = a * x0[r];
    for (i = 1; i < h; i++) {
      const double* xc = col(x, i);
      a = c[i + (long)j * gh];
      for (r = 0; r < x->n; r++) yc[r] += a * xc[r];
    }
  }
}

/* y(active) = d(mask) .* x(active): multi_vector.c:291-349 */
static void blk_bydiag(const blk* x, const int* mask, int k, const double* d, blk* y)
{
  int i, c = 0;
  long r;
  for (i = 0; i < k; i++) {
    if (mask && !mask[i]) continue;
    {
      const double* s = col(x, c);
      double* t = col(y, c);
      for (r = 0; r < x->n; r++) t[r] = d[i] * s[r];
    }
    c++;
  }
}

/* d(mask) = diag(x' y): multi_vector.c:411-469 */
static void blk_diaginner(const blk* x, const blk* y, const int* mask, int k, double* d)
{
  int i, c = 0;
  long r;
  for (i = 0; i < k; i++) {
    if (mask && !mask[i]) continue;
    {
      const double* a = col(x, c);
      const double* b = col(y, c);
      double s = 0.0;
      for (r = 0; r < x->n; r++) s += a[r] * b[r];
      d[i] = s;
    }
    c++;
  }
}

static void blk_apply(const oracle_op* op, const blk* x, blk* y)
{
  int c;
  for (c = 0; c < x->na; c++) op_apply_col(op, x->n, col(x, c), col(y, c));
}

/* ------------------------------------------------------------------ */
/* small column-major matrices (fortran_matrix.c)                     */
/* ------------------------------------------------------------------ */

/* (m + m')/2 on an m x m block: fortran_matrix.c:428-452 */
static void sm_symmetrize(double* a, int ld, int m)
{
  int i, j;
  for (j = 0; j < m; j++)
    for (i = j + 1; i < m; i++) {
      double v = (a[i + (long)j * ld] + a[j + (long)i * ld]) * 0.5;
      a[i + (long)j * ld] = v;
      a[j + (long)i * ld] = v;
    }
}

/* zero strictly-lower part: fortran_matrix.c:257-279 */
static void sm_clear_lower(double* a, int ld, int m)
{
  int i, j;
  for (j = 0; j < m; j++)
    for (i = j + 1; i < m; i++) a[i + (long)j * ld] = 0.0;
}

/* identity on an h x w block: fortran_matrix.c:313-330 */
static void sm_identity(double* a, int ld, int h, int w)
{
  int i, j;
  for (j = 0; j < w; j++)
    for (i = 0; i < h; i++) a[i + (long)j * ld] = (i == j) ? 1.0 : 0.0;
}

/* in-place inverse of an upper-triangular m x m block:
   fortran_matrix.c:1368-1416 (column-by-column back substitution) */
static void sm_upper_inv(double* u, int ld, int m)
{
  double* d = (double*)malloc(sizeof(double) * (m > 0 ? m : 1));
  int i, j, l;
  for (i = 0; i < m; i++) {
    d[i] = u[i + (long)i * ld];
    u[i + (long)i * ld] = 1.0 / d[i];
  }
  for (i = m - 2; i >= 0; i--)
    for (j = m - 1; j > i; j--) {
      double s = 0.0;
      for (l = i + 1; l <= j; l++) s -= u[i + (long)l * ld] * u[l + (long)j * ld];
      u[i + (long)j * ld] = s / d[i];
    }
  free(d);
}

/* c = op(a) * op(b): fortran_matrix.c:1016-1077 */
static void sm_multiply(const double* a, int lda, int ta, const double* b, int ldb, int tb,
                        double* c, int ldc, int h, int w, int l)
{
  int i, j, q;
  for (j = 0; j < w; j++)
    for (i = 0; i < h; i++) {
      double s = 0.0;
      for (q = 0; q < l; q++) {
        double av = ta ? a[q + (long)i * lda] : a[i + (long)q * lda];
        double bv = tb ? b[j + (long)q * ldb] : b[q + (long)j * ldb];
        s += av * bv;
      }
      c[i + (long)j * ldc] = s;
    }
}

/* ------------------------------------------------------------------ */
/* the solver                                                          */
/* ------------------------------------------------------------------ */

typedef struct {
  dsygv_fn sygv;
  dpotrf_fn potrf;
} lapack_t;

/* Host-side fault injection for the failure-path tests: the Nth call
   (1-based) of the Cholesky or of the generalized eigensolver reports
   INFO = 1.  0 disables.  Mirrors ref_set_faults in ref_harness.c. */
static int g_potrf_fail_at = 0, g_potrf_calls = 0;
static int g_sygv_fail_at = 0, g_sygv_calls = 0;

void oracle_set_faults(int potrf_fail_at, int sygv_fail_at)
{
  g_potrf_fail_at = potrf_fail_at;
  g_sygv_fail_at = sygv_fail_at;
}

/* lobpcg.c:20-39 (Cholesky, upper) */
static int chol_upper(const lapack_t* lp, double* a, int ld, int m)
{
  char uplo = 'U';
  int info = 0;
  lp->potrf(&uplo, &m, a, &ld, &info);
  if (++g_potrf_calls == g_potrf_fail_at && info == 0) info = 1;
  return info;
}

/* lobpcg.c:66-103 (dsygv itype 1, jobz V, uplo L, lwork 10 m) */
static int gevp(const lapack_t* lp, double* a, double* b, int ld, int m, double* w)
{
  int itype = 1, lwork = 10 * m, info = 0;
  char jobz = 'V', uplo = 'L';
  double* work;
  if (++g_sygv_calls == g_sygv_fail_at) return 1;
  work = (double*)calloc(lwork > 0 ? lwork : 1, sizeof(double));
  lp->sygv(&itype, &jobz, &uplo, &m, a, &ld, b, &ld, w, work, &lwork, &info);
  free(work);
  return info;
}

/* B-orthonormalise x (bx = B x) with r = chol(x'bx)^{-1}: lobpcg.c:197-232 */
static int implicit_qr(const lapack_t* lp, blk* x, const blk* bx, double* r, int ld, blk* z)
{
  int m = x->na, info;
  blk_gram(x, bx, ld, r);
  info = chol_upper(lp, r, ld, m);
  if (info != 0) return info;
  sm_upper_inv(r, ld, m);
  sm_clear_lower(r, ld, m);
  blk_copy(x, z);
  blk_bymat(z, ld, m, m, r, x);
  return 0;
}

/* lobpcg.c:237-260 */
static void residual_norms(const blk* r, double* norms, double* diag, const int* mask, int k)
{
  int i;
  blk_diaginner(r, r, mask, k, diag);
  for (i = 0; i < k; i++)
    if (mask == NULL || mask[i]) norms[i] = sqrt(fabs(diag[i]));
}

/* lobpcg.c:265-294 */
static int check_residuals(const double* norms, const double* lambda, double atol, double rtol,
                           int* mask, int k)
{
  int i, active = 0;
  for (i = 0; i < k; i++) {
    if (norms[i] > fabs(lambda[i]) * rtol + atol + DBL_EPSILON) {
      mask[i] = 1;
      active++;
    } else
      mask[i] = 0;
  }
  return active;
}

/*
 * oracle_solve: restates lobpcg_solve (lobpcg.c:502-1388) for real double
 * data.  x (n*k, column-major) is the initial block on entry and the Ritz
 * vectors on exit.  Operators: kind OP_NONE for "no B" / "no T".  y: ny
 * constraint columns or ny == 0.  Histories may be NULL; otherwise k x
 * (maxit+1) column-major with ld k.  Returns the reference's exit flag.
 */
int oracle_solve(long n, int k, oracle_op A, oracle_op B, oracle_op T,
                 int ny, const double* ydata, double* x,
                 double atol, double rtol, int maxit,
                 void* dsygv_ptr, void* dpotrf_ptr,
                 double* lambda, double* resnorm, double* lambda_hist, double* res_hist,
                 int* iterations)
{
  lapack_t lp;
  int noB = B.kind == OP_NONE, noT = T.kind == OP_NONE, noY = ny == 0;
  int exitflag = 0, it, i;
  int k3 = 3 * k;
  int sizeR = 0, sizeP = 0, sizeA, firstR, lastR, firstP;
  blk *X, *R, *P, *W, *AX, *AR, *AP, *BX, *BR, *BP, *Y = NULL, *BY = NULL;
  double *gA, *gB, *lamAB, *rdiag, *gYBY = NULL, *gYBX = NULL, *tYBX = NULL;
  int* mask;

  lp.sygv = (dsygv_fn)dsygv_ptr;
  lp.potrf = (dpotrf_fn)dpotrf_ptr;
  g_potrf_calls = 0;
  g_sygv_calls = 0;
  *iterations = 0;

  /* lobpcg.c:689-698 */
  if (k < 1) return 2;

  X = blk_new(n, k, x);
  W = blk_new(n, k, NULL);
  rdiag = (double*)calloc(k, sizeof(double));

  /* constraints: lobpcg.c:700-751 */
  if (!noY) {
    Y = blk_new(n, ny, (double*)ydata);
    gYBY = (double*)calloc((size_t)ny * ny, sizeof(double));
    gYBX = (double*)calloc((size_t)ny * k, sizeof(double));
    tYBX = (double*)calloc((size_t)ny * k, sizeof(double));
    BY = Y;
    if (!noB) {
      BY = blk_new(n, ny, NULL);
      blk_apply(&B, Y, BY);
    }
    blk_gram(BY, Y, ny, gYBY);
    if (chol_upper(&lp, gYBY, ny, ny) != 0) {
      if (!noB) blk_free(BY);
      blk_free(Y);
      blk_free(W);
      blk_free(X);
      free(gYBY); free(gYBX); free(tYBX); free(rdiag);
      return 3;
    }
    sm_upper_inv(gYBY, ny, ny);
    sm_clear_lower(gYBY, ny, ny);
    blk_gram(BY, X, ny, gYBX);
    sm_multiply(gYBY, ny, 1, gYBX, ny, 0, tYBX, ny, ny, k, ny);
    sm_multiply(gYBY, ny, 0, tYBX, ny, 0, gYBX, ny, ny, k, ny);
    blk_bymat(Y, ny, ny, k, gYBX, W);
    blk_axpy(-1.0, W, X);
  }

  gA = (double*)calloc((size_t)k3 * k3, sizeof(double));
  gB = (double*)calloc((size_t)k3 * k3, sizeof(double));
  lamAB = (double*)calloc(k3, sizeof(double));
  mask = (int*)malloc(sizeof(int) * k);
  for (i = 0; i < k; i++) mask[i] = 1;

  R = blk_new(n, k, NULL);
  P = blk_new(n, k, NULL);
  AX = blk_new(n, k, NULL);
  AR = blk_new(n, k, NULL);
  AP = blk_new(n, k, NULL);
  if (!noB) {
    BX = blk_new(n, k, NULL);
    BR = blk_new(n, k, NULL);
    BP = blk_new(n, k, NULL);
  } else {
    BX = X;
    BR = R;
    BP = P;
  }

  /* initial B-orthonormalisation and Rayleigh-Ritz: lobpcg.c:853-962 */
  if (!noB) blk_apply(&B, X, BX);
  exitflag = implicit_qr(&lp, X, BX, gB, k3, W);
  if (exitflag == 0) {
    if (!noB) {
      blk_bymat(BX, k3, k, k, gB, W);
      blk_copy(W, BX);
    }
    blk_apply(&A, X, AX);
    blk_gram(X, AX, k3, gA);
    sm_symmetrize(gA, k3, k);
    blk_gram(X, BX, k3, gB);
    sm_symmetrize(gB, k3, k);
    exitflag = gevp(&lp, gA, gB, k3, k, lambda);
    if (exitflag == 0) {
      blk_bymat(X, k3, k, k, gA, W);
      blk_copy(W, X);
      blk_bymat(AX, k3, k, k, gA, W);
      blk_copy(W, AX);
      if (!noB) {
        blk_bymat(BX, k3, k, k, gA, W);
        blk_copy(W, BX);
      }
      blk_bydiag(BX, NULL, k, lambda, R);
      blk_axpy(-1.0, AX, R);
      residual_norms(R, resnorm, rdiag, NULL, k);
      if (lambda_hist) memcpy(lambda_hist, lambda, sizeof(double) * k);
      if (res_hist) memcpy(res_hist, resnorm, sizeof(double) * k);
    }
  }

  /* main loop: lobpcg.c:965-1318 */
  for (it = 1; exitflag == 0 && it <= maxit; it++) {
    double* coord;
    sizeR = check_residuals(resnorm, lambda, atol, rtol, mask, k);
    if (sizeR < 1) break;
    blk_mask(R, mask);
    blk_mask(P, mask);
    blk_mask(AR, mask);
    blk_mask(AP, mask);
    if (!noB) {
      blk_mask(BR, mask);
      blk_mask(BP, mask);
    }
    blk_mask(W, mask);

    if (!noT) {
      blk_apply(&T, R, W);
      blk_copy(W, R);
    }

    if (!noY) {
      /* lobpcg.c:996-1012; gYBR/tYBR are the leading ny x sizeR blocks */
      blk_gram(BY, R, ny, gYBX);
      sm_multiply(gYBY, ny, 1, gYBX, ny, 0, tYBX, ny, ny, sizeR, ny);
      sm_multiply(gYBY, ny, 0, tYBX, ny, 0, gYBX, ny, ny, sizeR, ny);
      blk_bymat(Y, ny, ny, sizeR, gYBX, W);
      blk_axpy(-1.0, W, R);
    }

    firstR = k;          /* 0-based offsets of the R and P blocks */
    lastR = k + sizeR;   /* one past the end */
    firstP = lastR;

    if (!noB) blk_apply(&B, R, BR);
    exitflag = implicit_qr(&lp, R, BR, gB + firstR + (long)firstR * k3, k3, W);
    if (exitflag) break;
    if (!noB) {
      blk_bymat(BR, k3, sizeR, sizeR, gB + firstR + (long)firstR * k3, W);
      blk_copy(W, BR);
    }
    blk_apply(&A, R, AR);

    if (it > 1) {
      double* up;
      sizeP = sizeR;
      up = gB + firstP + (long)firstP * k3;
      exitflag = implicit_qr(&lp, P, BP, up, k3, W);
      if (exitflag) {
        sizeP = 0; /* lobpcg.c:1056-1063: steepest-descent restart */
      } else {
        if (!noB) {
          blk_bymat(BP, k3, sizeR, sizeR, up, W);
          blk_copy(W, BP);
        }
        blk_bymat(AP, k3, sizeR, sizeR, up, W);
        blk_copy(W, AP);
      }
    } else {
      sizeP = 0;
    }
    sizeA = lastR + sizeP;

    /* Gram blocks with the implicit identities: lobpcg.c:1092-1160 */
    sm_identity(gA, k3, k, k);
    for (i = 0; i < k; i++) gA[i + (long)i * k3] = lambda[i];
    blk_gram(R, AX, k3, gA + firstR);
    blk_gram(R, AR, k3, gA + firstR + (long)firstR * k3);
    sm_symmetrize(gA + firstR + (long)firstR * k3, k3, sizeR);
    sm_identity(gB, k3, k, k);
    blk_gram(R, BX, k3, gB + firstR);
    sm_identity(gB + firstR + (long)firstR * k3, k3, sizeR, sizeR);
    if (it > 1) {
      blk_gram(P, AX, k3, gA + firstP);
      blk_gram(P, AR, k3, gA + firstP + (long)firstR * k3);
      blk_gram(P, AP, k3, gA + firstP + (long)firstP * k3);
      sm_symmetrize(gA + firstP + (long)firstP * k3, k3, sizeR);
      blk_gram(P, BX, k3, gB + firstP);
      blk_gram(P, BR, k3, gB + firstP + (long)firstR * k3);
      sm_identity(gB + firstP + (long)firstP * k3, k3, sizeR, sizeR);
    }

    /* Rayleigh-Ritz: lobpcg.c:1164-1181 */
    exitflag = gevp(&lp, gA, gB, k3, sizeA, lamAB);
    if (exitflag != 0) {
      fprintf(stderr, "Return Code %d\n", exitflag);
      printf("INFO = %d\n", exitflag);
      it--;
      break;
    }
    memcpy(lambda, lamAB, sizeof(double) * k);
    coord = gA; /* coordX = gramA(1:sizeA, 1:k) */

    /* P, AP, BP and X, AX, BX updates: lobpcg.c:1191-1272.  For it > 1 the
       P coordinates are rows firstP..firstP+sizeR of gramA even when the
       P orthonormalisation failed (the reference keeps lastP unchanged). */
    if (it > 1) {
      blk_mask(W, NULL);
      blk_bymat(P, k3, sizeR, k, coord + firstP, W);
      blk_mask(P, NULL);
      blk_copy(W, P);
      blk_bymat(AP, k3, sizeR, k, coord + firstP, W);
      blk_mask(AP, NULL);
      blk_copy(W, AP);
      if (!noB) {
        blk_bymat(BP, k3, sizeR, k, coord + firstP, W);
        blk_mask(BP, NULL);
        blk_copy(W, BP);
      }
      blk_bymat(R, k3, sizeR, k, coord + firstR, W);
      blk_axpy(1.0, W, P);
      blk_bymat(AR, k3, sizeR, k, coord + firstR, W);
      blk_axpy(1.0, W, AP);
      if (!noB) {
        blk_bymat(BR, k3, sizeR, k, coord + firstR, W);
        blk_axpy(1.0, W, BP);
      }
    } else {
      blk_mask(P, NULL);
      blk_bymat(R, k3, sizeR, k, coord + firstR, P);
      blk_mask(AP, NULL);
      blk_bymat(AR, k3, sizeR, k, coord + firstR, AP);
      if (!noB) {
        blk_mask(BP, NULL);
        blk_bymat(BR, k3, sizeR, k, coord + firstR, BP);
      }
    }

    blk_mask(W, NULL);
    blk_copy(X, W);
    blk_bymat(W, k3, k, k, coord, X);
    blk_axpy(1.0, P, X);
    blk_copy(AX, W);
    blk_bymat(W, k3, k, k, coord, AX);
    blk_axpy(1.0, AP, AX);
    if (!noB) {
      blk_copy(BX, W);
      blk_bymat(W, k3, k, k, coord, BX);
      blk_axpy(1.0, BP, BX);
    }

    /* residuals of the active columns: lobpcg.c:1274-1286 */
    blk_mask(AX, mask);
    blk_mask(BX, mask);
    blk_bydiag(BX, mask, k, lambda, R);
    blk_axpy(-1.0, AX, R);
    residual_norms(R, resnorm, rdiag, mask, k);
    if (lambda_hist) memcpy(lambda_hist + (long)it * k, lambda, sizeof(double) * k);
    if (res_hist) memcpy(res_hist + (long)it * k, resnorm, sizeof(double) * k);

    blk_mask(AX, NULL);
    blk_mask(BX, NULL);
    blk_mask(AP, mask);
    blk_mask(BP, mask);
    blk_mask(P, mask);
    blk_mask(W, mask);
  }

  /* lobpcg.c:1321-1324 */
  if (exitflag != 0 || it > maxit) exitflag = -1;
  *iterations = it - 1;

  blk_free(R);
  blk_free(P);
  blk_free(AX);
  blk_free(AR);
  blk_free(AP);
  if (!noB) {
    blk_free(BX);
    blk_free(BR);
    blk_free(BP);
    if (!noY) blk_free(BY);
  }
  if (!noY) blk_free(Y);
  blk_free(W);
  blk_free(X);
  free(gA); free(gB); free(lamAB); free(rdiag); free(mask);
  free(gYBY); free(gYBX); free(tYBX);
  return exitflag;
}

/* Block operator application, exported for kernel-level checks:
   y(:, c) = op(x(:, c)) for c < k, column-major with ld n. */
void oracle_apply(long n, int k, oracle_op op, const double* x, double* y)
{
  int c;
  for (c = 0; c < k; c++) op_apply_col(&op, n, x + (long)c * n, y + (long)c * n);
}
