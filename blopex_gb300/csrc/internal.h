/*
 * internal.h -- shared declarations of the GB300 LOBPCG library (not part
 * of the public C ABI).  Included by the C host driver and the CUDA files.
 */
#ifndef BLOPEX_GB300_INTERNAL_H
#define BLOPEX_GB300_INTERNAL_H

#include <stddef.h>
#include "lobpcg_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* widest block handed to one kernel: [X R P] for k = 128 */
#define BLK_MAXCOLS 384
#define GB_POOL_MAX 64

/* Column pointer table passed by value to the block kernels: logical
   column c of an operand lives at col[c] (device address, `len` rows). */
typedef struct {
  const void* col[BLK_MAXCOLS];
} blk_cols;

/* kernel classes for the event timers */
enum {
  GB_K_GRAM = 0, GB_K_XC, GB_K_CSR, GB_K_ST7, GB_K_ST5, GB_K_ST27, GB_K_DIAG, GB_K_RESID,
  GB_K_BLAS1, GB_K_CHOLQR, GB_K_SYGV, GB_K_SMALL, GB_K_TC_GRAM, GB_K_TC_XC, GB_K_SYGV_FALLBACK,
  GB_K_RR_CHOL, GB_K_RR_TRSM, GB_K_RR_JAC32, GB_K_RR_GEMM, GB_K_RR_REFINE, GB_K_RR_TRID,
  GB_K_RR_EIG,
  /* the same operations with FP32 arithmetic (the mixed mode's FP32 phase) */
  GB_K_GRAM32, GB_K_XC32, GB_K_CSR32, GB_K_ST7_32, GB_K_ST5_32, GB_K_ST27_32, GB_K_DIAG32,
  /* FP64-accurate split-operand products on the tensor cores */
  GB_K_OZ_XC, GB_K_OZ_GRAM,
  GB_K_COUNT
};

typedef struct {
  void* start; /* cudaEvent_t */
  void* stop;
  int cls;
  double bytes, flops;
} gb_prof_rec;

struct gpu_Context {
  int device;
  void* stream;       /* cudaStream_t */
  int owns_stream;
  lobpcg_gpu_options opt;
  lobpcg_gpu_stats stats;
  char err[512];
  /* grow-only device scratch for split-k partials and small matrices */
  void* work;
  size_t work_bytes;
  /* pinned host staging for small device->host reads */
  void* pinned;
  size_t pinned_bytes;
  int num_sms;
  /* host-side fault injection counters (see lobpcg_gpu_options) */
  int potrf_calls;
  int sygv_calls;
  /* kernel timers */
  int profile;
  gb_prof_rec* prof_pending;
  int prof_npending, prof_cap;
  void** prof_pool; /* free cudaEvent_t */
  int prof_npool;
  lobpcg_gpu_kernel_time prof[GB_K_COUNT];
  /* device counters: [0] FP32 Jacobi sweeps, [1] largest refinement
     cluster, [2] FP64 fallback solves, [3] Rayleigh-Ritz calls, [4] graded
     pencils, [5] tensor-core kernel error word */
  int* dcount;
  /* device buffers of the solver's internal blocks, kept across solves (all
     work is ordered on ctx->stream, so a returned buffer can be handed out
     again at once); freed by gpu_ContextTrim / gpu_ContextDestroy */
  /* set around the FP32 phase's A R: FP32 blocks through CSR / 7-point
     operators with FP64 coefficients and arithmetic */
  int op_accurate;
  int pool_n;
  void* pool_ptr[GB_POOL_MAX];
  size_t pool_bytes[GB_POOL_MAX];
};

/* internal block storage from / back to the context's pool */
void* gb_pool_get(gpu_Context* ctx, size_t bytes);
void gb_pool_put(gpu_Context* ctx, void* p, size_t bytes);

/* error helpers (context.cu) */
int gb_fail(gpu_Context* ctx, const char* fmt, ...);
int gb_cuda_check(gpu_Context* ctx, int cuda_status, const char* what);
void* gb_workspace(gpu_Context* ctx, size_t bytes);
/* the CUDA driver's cuTensorMapEncodeTiled (operators.cu), NULL when absent */
void* gb_tensormap_encoder(void);
void* gb_pinned(gpu_Context* ctx, size_t bytes);
void gb_count_launch(long long n);
int gb_memcpy_d2h(gpu_Context* ctx, void* dst, const void* src, size_t bytes);
int gb_memcpy_h2d(gpu_Context* ctx, void* dst, const void* src, size_t bytes);
int gb_memcpy_d2d(gpu_Context* ctx, void* dst, const void* src, size_t bytes);
int gb_sync(gpu_Context* ctx);
void* gb_device_alloc(gpu_Context* ctx, size_t bytes);
void gb_device_free(void* p);
double gb_now(void);
/* bracket one kernel launch (no-ops unless profiling is on) */
void gb_prof_begin(gpu_Context* ctx, gb_prof_rec* rec, int cls);
void gb_prof_end(gpu_Context* ctx, gb_prof_rec* rec, double bytes, double flops);
/* fold finished timers into ctx->prof (synchronises the stream) */
void gb_prof_collect(gpu_Context* ctx);

/* multivector helpers (multivector.cu) */
int gb_is_gpu_interpreter(const mv_InterfaceInterpreter* ii);
void gb_mv_set_mask_host(gpu_MultiVector* x, const BlopexInt* mask);
int gb_mv_sync_mask(gpu_MultiVector* x);
gpu_MultiVector* gb_mv_create_like(const gpu_MultiVector* x, int dtype);
int gb_mv_fill_cols(const gpu_MultiVector* x, blk_cols* t, int offset);

/* ---------------- block kernels (blockops.cu) ---------------- */
/* G(0:h,0:w) (column-major, leading dimension ldg, FP64, device) =
   X(:,0:h)' * Y(:,0:w); X and Y share dtype. */
int gb_gram(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h, const blk_cols* Y,
            int w, double* G, int ldg);
/* Y(:,j) = sum_i X(:,i) C(i,j) [+ Z(:,j)], C FP64 device column-major (ldc) */
int gb_bymat(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h, const double* C,
             int ldc, const blk_cols* Y, int w, const blk_cols* Z);
/* the same with C upper triangular (explicit zeros below the diagonal) */
int gb_bymat_tri(gpu_Context* ctx, int dtype, long n, const blk_cols* X, int h, const double* C,
                 int ldc, const blk_cols* Y, int w);
/* Y(:,j) = alpha * X(:,j) + beta * Y(:,j) for j < w */
int gb_axpby(gpu_Context* ctx, int dtype, long n, double alpha, const blk_cols* X, double beta,
             const blk_cols* Y, int w);
/* Y(:,j) = d[idx[j]] * X(:,j) (d FP64 device; idx host) */
int gb_scale_cols(gpu_Context* ctx, int dtype, long n, const blk_cols* X, const double* d,
                  const int* idx, const blk_cols* Y, int w);
/* out[idx[j]] = X(:,j)' Y(:,j) (FP64 device) */
int gb_dot_cols(gpu_Context* ctx, int dtype, long n, const blk_cols* X, const blk_cols* Y, int w,
                double* out, const int* idx);
/* the fixed-order sum of per-CTA partials partial[j * nb + b] into
   out[idx[j]], and the row-block count the column kernels use */
int gb_dot_reduce(gpu_Context* ctx, const double* partial, int nb, int w, double* out,
                  const int* idx);
unsigned gb_row_blocks(gpu_Context* ctx, long n, int w);
/* Y(:,j) (dtype_y) = X(:,j) (dtype_x), converting precision */
int gb_convert(gpu_Context* ctx, long n, int dtype_x, const blk_cols* X, int dtype_y,
               const blk_cols* Y, int w);
/* fused residual: R(:,j) = lambda[idx[j]] * BX(:,j) - AX(:,j); norm2[idx[j]] = |R(:,j)|^2.
   dtype GB_RESID_64TO32: FP64 BX, AX and an FP32 R (norms from the FP64 values) */
#define GB_RESID_64TO32 3
int gb_residual(gpu_Context* ctx, int dtype, long n, const blk_cols* BX, const blk_cols* AX,
                const double* lambda, const int* idx, const blk_cols* R, int w, double* norm2);
/* Y64 = X64 + D32 and D32 <- (float) Y64, columnwise */
int gb_accumulate64(gpu_Context* ctx, long n, const blk_cols* X64, const blk_cols* D32,
                    const blk_cols* Y64, int w);
/* lam[j] = X(:,j)'AX(:,j) / X(:,j)'X(:,j) (device; scratch: 2w doubles) */
int gb_rayleigh_quotients(gpu_Context* ctx, int dtype, long n, const blk_cols* X,
                          const blk_cols* AX, int w, double* scratch, double* lam);
/* Cholesky with deflation of columns whose pivot ratio is below tol; A <-
   inv(U) with the dropped columns zeroed; dropped[j] (device) marks them,
   *ndrop (device) counts them */
int gb_chol_deflate(gpu_Context* ctx, double* A, int ld, int m, double tol, int* dropped, int* ndrop);
/* decouple the dropped coordinates off + j of a pencil (H2_jj = 1, G2_jj above
   the kx smallest eigenvalues) */
int gb_deflate_pencil(gpu_Context* ctx, double* G, double* H, int ld, int mtot, int off, int m,
                      const int* dropped, int kx);
/* the explicit pencil (G, H; m x m, m = k + nR + nP, leading dimension ld)
   of the split mode from Hx = X'[X R P] (ld k), Hr = R'[R P AR AP] (ld nR),
   Hp = P'[P AP] (ld nP), Gt = RS'[RS S] (ld k: S_c' RS_i at Gt[i + (k + c) k];
   RS = lambda X - A X) and
   lambda: the X rows of G in residual form, lambda_i X_i'S_c - RS_i'S_c */
int gb_split_pencil(gpu_Context* ctx, const double* Hx, const double* Hr, const double* Hp,
                    const double* Gt, double* G, double* H, int ld, const double* lam, int k,
                    int nR, int nP);
/* A(i,i) += alpha for i < m (device small matrix) */
int gb_small_add_diag(gpu_Context* ctx, double* A, int ld, int m, double alpha);
/* drand48-compatible fill of column-major storage, columns listed in idx */
int gb_drand48_fill(gpu_Context* ctx, int dtype, void* data, long n, long ld, const int* idx,
                    int w, unsigned int seed);

/* tensor-core Gram of the explicit iteration (tc_gram.cu): FP32 blocks X (k
   columns), R (nR), P (nP) and their images AX, AR, AP; k <= 64, nR, nP <=
   32 (k <= 32) or 64.  G = [X R P]'[AX AR AP], H = [X R P]'[X R P] (m x m,
   m = k + nR + nP, FP64, leading dimension ld).  compensated: 3xTF32. */
int gb_tc_gram(gpu_Context* ctx, long n, const blk_cols* X, int k, const blk_cols* R, int nR,
               const blk_cols* P, int nP, const blk_cols* AX, const blk_cols* AR,
               const blk_cols* AP, int compensated, double* G, double* H, int ld);

/* Y = X C (+ Z) on the tensor cores, compensated TF32 (tc_xc.cu): FP32
   columns, h <= 128, w <= 64, C FP64 on the device (leading dimension ldc) */
int gb_tc_xc(gpu_Context* ctx, long n, const blk_cols* X, int h, const double* C, int ldc,
             const blk_cols* Y, int w, const blk_cols* Z);
/* FP64-accurate Y = X C (+ Z) on the tensor cores by error-free splitting
   (oz_xc.cu): X FP64 (h <= 64 columns, 16-byte aligned, readable up to an
   even row count), C FP64 device (ldc), Y FP64 (w <= 64); Z optional, FP32
   or FP64 (z_dtype); Y32 optional FP32 copy of Y */
int gb_oz_xc(gpu_Context* ctx, long n, const blk_cols* X, int h, const double* C, int ldc,
             const blk_cols* Y, int w, const blk_cols* Z, int z_dtype, const blk_cols* Y32);
/* FP64-accurate Gram G = L' [L Q_0 Q_1 ...] on the tensor cores (oz_gram.cu):
   L a block of h <= 64 columns, FP32 or FP64 (ldt); nq <= 4 blocks Q_b of up
   to 64 columns each, FP32 or FP64 (qdt[b]); every column 16-byte aligned and
   readable up to a row count rounded to 4.  G (FP64 device, ldg) receives L'L
   in columns 0..h and L'Q_b in the following columns, in order. */
int gb_oz_gram(gpu_Context* ctx, long n, const blk_cols* L, int h, int ldt, int nq,
               const blk_cols* Q, const int* qw, const int* qdt, double* G, int ldg);
/* device error word of the tensor-core kernels (0 = none); clears it */
int gb_device_error(gpu_Context* ctx, int* err);

/* ---------------- small dense FP64 (dense.cu) ---------------- */
/* in place: A(0:m,0:m) upper Cholesky factor U (A = U'U from the upper
   triangle), then A <- inv(U) with the strict lower part cleared; *info
   (device int) = 0 or the order of the first non-positive leading minor */
int gb_cholqr_factor(gpu_Context* ctx, double* A, int ld, int m, int* info);
/* generalized symmetric-definite eigenproblem A v = w B v (itype 1, lower
   triangles read): A <- eigenvectors (B-orthonormal, ascending), w <- values,
   B <- its lower Cholesky factor; *info as dsygv */
/* Rayleigh-Ritz: lowest nev eigenpairs of A v = w B v into A's first nev
   columns and w; INFO as dsygv.  B is reported as not definite (INFO m+j)
   when a Cholesky pivot ratio L_jj^2 / B_jj falls below report_below. */
int gb_sygv(gpu_Context* ctx, double* A, double* B, int ld, int m, int nev, double* w, int* info,
            double report_below);
/* small helpers on device matrices */
int gb_small_symmetrize(gpu_Context* ctx, double* A, int ld, int m);
int gb_small_identity(gpu_Context* ctx, double* A, int ld, int h, int w);
int gb_small_diag(gpu_Context* ctx, double* A, int ld, int m, const double* d);
/* B(0:h,0:w) = A(0:h,0:w) */
int gb_small_copy(gpu_Context* ctx, const double* A, int lda, double* B, int ldb, int h, int w);
/* C(0:h,0:w) = op(A) op(B), inner dimension l (constraints path) */
int gb_small_gemm(gpu_Context* ctx, const double* A, int lda, int ta, const double* B, int ldb,
                  int tb, double* C, int ldc, int h, int w, int l);

/* explicit-Gram Rayleigh-Ritz helpers: d = 1/sqrt(diag H), Gs = D sym(G) D,
   Hs = D sym(H) D (unit diagonal); then C(0:m,0:k) <- D C */
int gb_scale_pencil(gpu_Context* ctx, const double* G, const double* H, double* Gs, double* Hs,
                    double* d, int ld, int m);
int gb_scale_rows(gpu_Context* ctx, double* C, const double* d, int ld, int m, int k);

/* ---------------- operators (operators.cu) ---------------- */
struct gpu_Operator;
int gb_operator_apply(struct gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y);
/* Y = A X with dot_out[c] = X_c' Y_c (device, one per active column) folded
   into the operator's kernel: 0, or 1 when the operator cannot (nothing was
   done), -1 on an error */
int gb_operator_apply_dot(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* Y,
                          double* dot_out);

#ifdef __cplusplus
}
#endif

#endif
