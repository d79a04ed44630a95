/*
 * lobpcg_gb300.h -- the GB300 (sm_103a) backend behind the BLOPEX C API.
 *
 * Replaces the serial-double backend of the reference:
 *   serial_Multi_Vector (blopex_serial_double/multivector/multi_vector.h:22-32)
 *       -> gpu_MultiVector, a device-resident column-major n x k block;
 *   SerialSetupInterpreter (blopex_serial_double/pcg_multi/pcg_multi.c:207-242)
 *       -> GpuSetupInterpreter;
 *   MatMultiVec / serial_Lapl1DMatMultiVec (pcg_multi.c:167-193,
 *   matmultivec.c:11-48) -> the device operators below (CSR SpMM, matrix-free
 *       7-point / 5-point / 27-point stencils, diagonal scaling for Jacobi T
 *       and lumped-mass B).
 * No torch or CUDA types appear here: streams are passed as void*
 * (a cudaStream_t), device memory as void*.
 */
#ifndef BLOPEX_GB300_H
#define BLOPEX_GB300_H

#include "lobpcg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- */
/* context: device, stream, solver options, statistics               */
/* ---------------------------------------------------------------- */

typedef struct gpu_Context gpu_Context;

enum { LOBPCG_GPU_FP64 = 0, LOBPCG_GPU_MIXED = 1 };
enum { GPU_MV_FLOAT64 = 0, GPU_MV_FLOAT32 = 1 };

typedef struct {
  int precision;            /* LOBPCG_GPU_FP64 (default) or LOBPCG_GPU_MIXED */
  double compensated_below; /* mixed: hi+lo compensated Gram once max residual < this (1e-6) */
  double fp64_below;        /* mixed: continue in FP64 once max residual < this (0: only on
                               convergence, stagnation or a failed factorisation) */
  int fp32_stall;           /* mixed: also switch after this many FP32 iterations without a
                               new minimum of the largest active residual (20) */
  int tensor_cores;         /* mixed: 1 = tcgen05 TF32 kernels, 0 = FP32 CUDA-core kernels */
  int potrf_fail_at;        /* tests: the Nth Cholesky reports INFO = 1 (0 = off) */
  int sygv_fail_at;         /* tests: the Nth Rayleigh-Ritz solve reports INFO = 1 (0 = off) */
  double explicit_pivot_below; /* mixed FP32 phase: P is dropped when a Cholesky pivot ratio of the
                               projected Gram matrix falls below this (1e-6: the FP32 Gram
                               products do not resolve smaller angles) */
  int fp32_accurate_op;      /* mixed FP32 phase: apply A to the residual block with FP64
                               coefficients and arithmetic (CSR and 7-point operators; 0) */
  int recompute_ap;          /* mixed FP32 phase: A P applied to the new P instead of updated
                               from [AR AP] (1) */
  int explicit_fp64;        /* diagnostics: run the mixed mode's explicit-Gram phase on FP64
                               blocks (CUDA-core kernels), to separate algorithm from precision */
  int accum64;              /* mixed, tensor-core path: carry X and A X in FP64 through the FP32
                               phase, adding FP32 corrections (0: measured no faster to 1e-8,
                               and its FP64 streams cost ~40 % per FP32 iteration) */
  int rr_method;            /* Rayleigh-Ritz solver: 0 = FP64 Householder tridiagonalisation,
                               bisection and inverse iteration (default); 1 = one-CTA FP64
                               Jacobi; 2 = FP32 Jacobi + FP64 refinement (order <= 192).
                               1 is also the fallback of 0 and 2. */
  int fp32_precond;         /* mixed: the inner-CG preconditioner (gpu_PCGPreconditionerCreate)
                               iterates on FP32 copies of FP64 blocks (the FP64 phase); the
                               preconditioner only shapes the search directions (0) */
  int split_products;       /* mixed, tensor-core path (B = I, no constraints, k <= 64): carry X
                               and A X in FP64 and form the products that decide the final
                               residual FP64-accurately on the tensor cores (split-operand X C
                               updates and X' [X R P] Gram rows), so the explicit phase itself
                               iterates to the tolerance (1) */
  int wait_polls;           /* tests: polls of one bounded pipeline wait in the tcgen05 / TMA
                               kernels before the wait gives up (error word, NaN output or the
                               step undone); 0 = the default 2^24.  The limit is held per
                               process and follows the last context that launched */
} lobpcg_gpu_options;

typedef struct {
  int iterations_fp32;      /* mixed: iterations run in FP32 storage */
  int iterations_fp64;      /* iterations run in FP64 storage */
  int iterations_compensated;
  long long kernel_launches;/* launches of this library's kernels during the last solve */
  double seconds_total;     /* wall time of the last solve (host clock, synchronised) */
  double seconds_fp32;
  double seconds_fp64;
  double final_max_residual;
  int rr_calls;             /* Rayleigh-Ritz solves of the last solve */
  int rr_jacobi32_sweeps;   /* FP32 Jacobi sweeps summed over those solves */
  int rr_max_cluster;       /* largest cluster of close Ritz values refined together */
  int rr_fallbacks;         /* solves that fell back to the one-CTA FP64 Jacobi */
  int rr_graded;            /* of those: pencils too graded for the tridiagonal solver */
  int explicit_undos;       /* mixed: FP32 steps undone after a residual jump */
  int explicit_p_drops;     /* mixed: FP32 steps taken without P (not definite / unresolved) */
  int iterations_split;     /* mixed: explicit-phase iterations with FP64-carried X (split
                               products) */
  int handover_reason;      /* mixed: why the explicit phase handed over to the FP64 loop:
                               0 it did not (converged or maxit), 1 residual below fp64_below,
                               2 no progress, 3 block not definite, 4 Rayleigh-Ritz failed,
                               5 residual jumps not repaired by undoing the step, 6 a
                               tensor-core or TMA kernel gave up waiting (its output is NaN) */
  int device_errors;        /* tensor-core kernels that reported a timed-out wait */
} lobpcg_gpu_stats;

/* per-kernel-class timing, collected with CUDA events on the context's
   stream when profiling is on (off by default) */
typedef struct {
  char name[24];
  long long launches;
  double ms;      /* summed event-timed duration */
  double bytes;   /* summed algorithmic bytes (operands read + results written once) */
  double flops;   /* summed algorithmic flops */
} lobpcg_gpu_kernel_time;

/* device < 0: current device.  stream == NULL: the library creates its own
   non-blocking stream.  Returns NULL on failure. */
gpu_Context* gpu_ContextCreate(int device, void* stream);
void gpu_ContextDestroy(gpu_Context* ctx);
void* gpu_ContextStream(gpu_Context* ctx);
int gpu_ContextSynchronize(gpu_Context* ctx);
/* free the device storage the context keeps for the solver's internal blocks
   between solves (it reuses it when the next solve has the same shapes) */
void gpu_ContextTrim(gpu_Context* ctx);
void gpu_ContextGetOptions(gpu_Context* ctx, lobpcg_gpu_options* opt);
int gpu_ContextSetOptions(gpu_Context* ctx, const lobpcg_gpu_options* opt);
void gpu_ContextGetStats(gpu_Context* ctx, lobpcg_gpu_stats* stats);
/* kernel timers: on/off, read (returns the number of classes written),
   reset */
int gpu_ContextSetProfiling(gpu_Context* ctx, int on);
int gpu_ContextKernelTimes(gpu_Context* ctx, lobpcg_gpu_kernel_time* out, int max);
void gpu_ContextResetKernelTimes(gpu_Context* ctx);
/* last error message of this context ("" if none) */
const char* gpu_ContextLastError(gpu_Context* ctx);
/* the device error word, read and cleared (waits for the context's stream):
   *code != 0 when a tcgen05 / TMA kernel gave up a bounded wait since the
   last read (its output holds NaN); returns nonzero on a CUDA error */
int gpu_ContextDeviceError(gpu_Context* ctx, int* code);
/* kernels launched by this library since it was loaded (all contexts) */
long long gpu_KernelLaunchCount(void);

/* ---------------------------------------------------------------- */
/* device multivector                                                */
/* ---------------------------------------------------------------- */

typedef struct {
  void* data;            /* device memory; column j starts at data + j*ld elements */
  long size;             /* rows n */
  long ld;               /* leading dimension in elements (>= size, multiple of 32) */
  BlopexInt num_vectors; /* columns k */
  BlopexInt dtype;       /* GPU_MV_FLOAT64 or GPU_MV_FLOAT32 */
  BlopexInt owns_data;
  BlopexInt num_active;  /* active columns (the mask) */
  BlopexInt* active;     /* host array: indices of the active columns, ascending */
  BlopexInt* active_dev; /* device copy of `active` */
  gpu_Context* ctx;
} gpu_MultiVector;

gpu_MultiVector* gpu_MultiVectorCreate(gpu_Context* ctx, long n, BlopexInt k, BlopexInt dtype);
/* wrap caller-owned device memory (not freed by Destroy) */
gpu_MultiVector* gpu_MultiVectorWrapDevice(gpu_Context* ctx, void* data, long n, long ld,
                                           BlopexInt k, BlopexInt dtype);
void gpu_MultiVectorDestroy(gpu_MultiVector* x);
/* whole-block host transfers, host column-major doubles with leading dimension ldh */
int gpu_MultiVectorFromHost(gpu_MultiVector* x, const double* host, long ldh);
int gpu_MultiVectorToHost(gpu_MultiVector* x, double* host, long ldh);
/* dst(:, all columns) = src(:, all columns), converting FP64 <-> FP32 */
int gpu_MultiVectorCopy(gpu_MultiVector* src, gpu_MultiVector* dst);
/* active columns = 2*drand48()-1 after srand48(seed), bit-identical to
   serial_Multi_VectorSetRandomValues (multi_vector.c:165-184) */
int gpu_MultiVectorSetRandomValues(gpu_MultiVector* x, BlopexInt seed);
/* fill `ii` with the device entries (the GPU counterpart of SerialSetupInterpreter) */
BlopexInt GpuSetupInterpreter(mv_InterfaceInterpreter* ii);

/* ---------------------------------------------------------------- */
/* operators: callbacks with the reference signature op(data, X, Y)  */
/* X, Y: gpu_MultiVector*; Y(active) = op(X(active)); FP64 or FP32   */
/* ---------------------------------------------------------------- */

typedef struct gpu_Operator gpu_Operator;

/* CSR with int32 column indices; host arrays are copied to the device */
gpu_Operator* gpu_CSRMatrixCreate(gpu_Context* ctx, long n, long nnz, const int* rowptr,
                                  const int* colidx, const double* vals);
/* 3D 7-point variable coefficient, Dirichlet: face coefficients
   cx[(k*ny + j)*(nx+1) + i] for the x-face between cells i-1 and i, likewise
   cy[(k*(ny+1) + j)*nx + i] and cz[(k*ny + j)*nx + i]; cells i + nx*(j + ny*k);
   (A x)_c = shift x_c + sum_f c_f (x_c - x_neighbour), x = 0 outside. */
gpu_Operator* gpu_Stencil7Create(gpu_Context* ctx, int nx, int ny, int nz, const double* cx,
                                 const double* cy, const double* cz, double shift);
/* 2D 5-point variable coefficient: cx[j*(nx+1) + i], cy[j*nx + i] */
gpu_Operator* gpu_Stencil5Create(gpu_Context* ctx, int nx, int ny, const double* cx,
                                 const double* cy, double shift);
/* 3D 27-point graph Laplacian + shift: w[13*c + e] is the weight of the edge
   from cell c to its forward neighbour e (offsets in the order
   (1,0,0) (-1,1,0) (0,1,0) (1,1,0) (-1,-1,1) (0,-1,1) (1,-1,1) (-1,0,1)
   (0,0,1) (1,0,1) (-1,1,1) (0,1,1) (1,1,1), as (di,dj,dk)); edges that leave
   the grid do not exist. */
gpu_Operator* gpu_Stencil27Create(gpu_Context* ctx, int nx, int ny, int nz, const double* w,
                                  double shift);
/* y = d .* x (Jacobi T with d = 1/diag(A); lumped mass B with d = diag(B)) */
gpu_Operator* gpu_DiagonalCreate(gpu_Context* ctx, long n, const double* d);
/* diag(A) of an operator, as host doubles (for building Jacobi T) */
int gpu_OperatorDiagonal(gpu_Operator* op, double* host_diag);
void gpu_OperatorDestroy(gpu_Operator* op);
/* the callback to pass as operatorA/B/T together with the gpu_Operator* */
void gpu_OperatorApply(void* op, void* X, void* Y);

/* Inner conjugate-gradient preconditioner T ~ inv(A): applying it runs
   `iterations` steps of CG on A Y = X from Y = 0, preconditioned by M (e.g.
   gpu_DiagonalCreate of 1/diag(A); may be NULL), every column independently
   and all columns in lockstep; in the dtype of the blocks.  The counterpart
   of the CG-preconditioned LOBPCG of HYPRE's driver (-pcgitr,
   blopex_hypre/krylov/HYPRE_lobpcg.c:317-320).  A and M must outlive it. */
gpu_Operator* gpu_PCGPreconditionerCreate(gpu_Context* ctx, gpu_Operator* A, gpu_Operator* M,
                                          int iterations);

/* The two Gram matrices of an explicit-Gram LOBPCG step on the active
   columns of the blocks: G = [X R P]'[AX AR AP], H = [X R P]'[X R P], m x m
   (m = widths of X + R + P; R/P and AR/AP may be NULL), written to host
   column-major arrays with leading dimension ldh.  mode 0: CUDA-core kernel
   (FP64 or FP32 blocks); mode 1: tensor cores, TF32 products with FP32
   accumulation; mode 2: tensor cores, compensated 3xTF32 (hi*hi + hi*lo +
   lo*hi); modes 1-2 take FP32 blocks with X at most 64 columns and R, P at
   most 32 (X <= 32) or 64 columns.  No counterpart in the reference, whose
   solver forms these blocks one pair at a time (lobpcg.c:1092-1160). */
int gpu_ExplicitGram(gpu_MultiVector* X, gpu_MultiVector* R, gpu_MultiVector* P,
                     gpu_MultiVector* AX, gpu_MultiVector* AR, gpu_MultiVector* AP, int mode,
                     double* G_host, double* H_host, int ldh);

/* Y(active) = X(active) C (+ Z(active)) for a host h x w column-major C
   (leading dimension ldc; h, w = active widths of X and Y); the operation of
   mv_MultiVectorByMatrix / serial_Multi_VectorByMatrix
   (blopex_serial_double/multivector/multi_vector.c:474-524) with the fused
   accumulate of the solver's X update.  mode 0: CUDA-core kernel (FP64 or FP32
   blocks); mode 1: tensor cores, compensated 3xTF32 (FP32 blocks, h <= 128,
   w <= 64, 16-byte aligned columns); mode 2: tensor cores, FP64-accurate
   products by error-free splitting into bf16 digits (FP64 X and Y, h <= 64,
   w <= 64; Z FP32 or FP64).  Z may be NULL. */
int gpu_BlockUpdate(gpu_MultiVector* X, const double* C_host, int ldc, gpu_MultiVector* Y,
                    gpu_MultiVector* Z, int mode);

/* G = L' [L Q_0 .. Q_{nq-1}] over the active columns, FP64-accurate on the
   tensor cores (error-free splitting of 64-row chunks into bf16 digits,
   exact FP32 accumulation per chunk, unbiased sums across chunks): L FP32 or
   FP64 with at most 64 active columns, each Q_b FP32 or FP64 with at most 64
   (nq <= 4).  G_host (h x (h + sum of the Q widths), leading dimension ldg)
   receives L'L and then each L'Q_b.  The Gram blocks of the reference's
   gramA / gramB (serial_Multi_VectorInnerProd, multi_vector.c:354-406, at
   lobpcg.c:1092-1160) as the mixed mode forms them.  Range: the chunk sums
   are scaled and accumulated in FP32 pairs, so the accuracy holds while, in
   every 64-row chunk, the product of two columns' largest magnitudes lies
   between 2^-120 and 2^100 (for instance every entry within [2^-60, 2^50]
   in magnitude; the solver's blocks -- unit columns and their images -- are
   well inside).  Outside it entries lose accuracy or overflow; a column
   whose chunk maximum is below 2^-118 or at least 2^135 counts as zero in
   that chunk. */
int gpu_SplitGram(gpu_MultiVector* L, gpu_MultiVector** Q, int nq, double* G_host, int ldg);

/* ---------------------------------------------------------------- */
/* External problems: the reference tools' file formats                */
/* ---------------------------------------------------------------- */

/* Host readers (no GPU work).  HYPRE IJ matrix files <prefix>.00000 ...
   (blopex_tools/matlab/matlab2hypre/matlab2hypreIJ.m: header "ilower iupper
   jlower jupper", then 0-based "row col value" triples) into CSR arrays;
   multivector text "n k" + values column by column (serial_Multi_VectorLoad,
   blopex_serial_complex/multivector/multi_vector.c:668-700): one value per
   entry, or the loader's (real, imaginary) pairs with zero imaginary parts;
   HYPRE ParVector files <prefix>.j.i (matlab2hypreParVectors.m: row count,
   then values) into a column-major n x k array.  Arrays are malloc'ed: free
   them with gpu_FreeHost.  Return 0, -1 (a file does not open), -2 (bad or
   short contents), -3 (index out of range), -4 (out of memory), -5 (a
   nonzero imaginary part in a multivector file). */
int gpu_ReadHypreIJ(const char* prefix, int nfiles, long* n, long* nnz, int** rowptr,
                    int** colidx, double** vals);
int gpu_ReadMultiVector(const char* path, long* n, int* k, double** data);
int gpu_ReadHypreParVectors(const char* prefix, int k, int nfiles, long* n, double** data);
void gpu_FreeHost(void* p);

/* The same, uploaded: a CSR operator, or a device block of the given dtype. */
gpu_Operator* gpu_CSRMatrixLoadHypreIJ(gpu_Context* ctx, const char* prefix, int nfiles);
gpu_MultiVector* gpu_MultiVectorLoad(gpu_Context* ctx, const char* path, int dtype);
gpu_MultiVector* gpu_MultiVectorLoadHypreParVectors(gpu_Context* ctx, const char* prefix, int k,
                                                    int nfiles, int dtype);

/* ---------------------------------------------------------------- */
/* Derivatives of the computed eigenpairs (no counterpart in the      */
/* reference)                                                          */
/* ---------------------------------------------------------------- */

/* Reverse mode for A x_i = lambda_i B x_i, X'BX = I (X: the n x k Ritz
   vectors returned by lobpcg_solve_double, FP64).  Given G = dL/dX (n x k
   FP64 block, or NULL) and glam = dL/dlambda (host k doubles, or NULL),
   writes W (n x k FP64): w_i = glam_i x_i + mu_i with
   mu_i = sum_{j != i} x_j (x_j'g_i) / (lambda_i - lambda_j) over the whole
   spectrum: the part inside span(X) explicitly (pairs closer than
   1e-12 max|lambda| are skipped), the rest by preconditioned conjugate
   gradients on (A - lambda_i B) restricted to the B-orthogonal complement of
   span(X), all columns in lockstep, until |r_i| <= tol |b_i| or maxit steps.
   A, B, T are operator callbacks as in lobpcg_solve_double (B, T may be NULL;
   T approximates the inverse of A).  xg (host k, may be NULL) receives
   g_i'x_i for gpu_MassGradient.  Returns 0 or -1 (message:
   gpu_ContextLastError); *iterations and *max_rel_residual report the solve. */
int gpu_EigenvectorAdjoint(gpu_MultiVector* X, const double* lambda, gpu_MultiVector* G,
                           const double* glam, void* Adata, void (*A)(void*, void*, void*),
                           void* Bdata, void (*B)(void*, void*, void*), void* Tdata,
                           void (*T)(void*, void*, void*), double tol, int maxit,
                           gpu_MultiVector* W, double* xg, int* iterations,
                           double* max_rel_residual);

/* Number of parameters of an operator: CSR nnz values; 7-point faces
   (cx | cy | cz concatenated, the layouts of gpu_Stencil7Create); 5-point
   faces (cx | cy); 27-point edge weights (cell-major n x 13, as passed to
   gpu_Stencil27Create); diagonal n. */
long gpu_OperatorParameterCount(gpu_Operator* op);

/* grad (host, gpu_OperatorParameterCount doubles) = sum_i w_i' (dA/dtheta)
   x_i for every parameter theta of A: with W from gpu_EigenvectorAdjoint this
   is dL/dtheta through the eigenpairs (dlambda_i/dA = x_i x_i' on the CSR
   pattern; a coupling c between cells p, q gives (w_p - w_q)(x_p - x_q),
   a boundary face w_p x_p).  The shift is not a parameter. */
int gpu_OperatorGradient(gpu_Operator* op, gpu_MultiVector* X, gpu_MultiVector* W,
                         double* grad);

/* grad (host, n) = dL/d(diagonal of B) for B = gpu_DiagonalCreate:
   -sum_i lambda_i w_i o x_i - (1/2) sum_i xg_i x_i o x_i (xg may be NULL). */
int gpu_MassGradient(gpu_Operator* B, gpu_MultiVector* X, gpu_MultiVector* W,
                     const double* lambda, const double* xg, double* grad);

/* ---------------------------------------------------------------- */
/* Gram product without any allocation                               */
/* ---------------------------------------------------------------- */

/*
 * G(0:h, 0:w) = X(:, 0:h)' * Y(:, 0:w) for column-major device blocks X
 * (leading dimension ldx) and Y (ldy) of n rows, both FP64 (dtype
 * GPU_MV_FLOAT64) or both FP32 (GPU_MV_FLOAT32); G is FP64 device memory with
 * leading dimension ldg; the kernels run on `stream` (a cudaStream_t).
 *
 * This entry point has no counterpart in the reference.  It is the same
 * split-k Gram kernel as the solver's (and as mv_MultiVectorByMultiVector
 * through the GPU interpreter), for callers that cannot allocate device
 * memory on this path: code running inside another framework's memory
 * pool that forbids raw cudaMalloc, or latency-critical code that must not
 * trigger the device synchronisation cudaMalloc/cudaFree can cause.  It
 * calls no cudaMalloc, cudaFree or allocating library routine; the split-k
 * partial sums go to one fixed device array of GPU_GRAM_NOALLOC_MAX_DOUBLES
 * doubles (4 MiB) that every GPU which loads the library holds until exit.
 *   - h and w must not exceed 384 (so h * w stays below that maximum); larger
 *     sizes are rejected with return value -2 (nothing is launched).
 *   - The first call on a device looks the array's address up
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture.
 *   - All calls share the array: calls that overlap on the GPU (concurrent
 *     streams, or several host threads) race on it and must be serialised
 *     by the caller.  The array keeps the last call's partial sums; every
 *     call overwrites all partials it reads, so nothing needs clearing.
 * Returns 0 on success, -1 for bad arguments, -2 for sizes beyond the
 * maximum, -3 for a CUDA error (also when an error from earlier work on the
 * calling thread is still pending; that error is left in place for its
 * owner and nothing is launched).
 */
#define GPU_GRAM_NOALLOC_MAX_DOUBLES (512 * 1024)
int gpu_GramNoAlloc(int dtype, long n, const void* X, long ldx, int h, const void* Y, long ldy,
                    int w, double* G, int ldg, void* stream);

#ifdef __cplusplus
}
#endif

#endif
