// multivector.cu -- gpu_MultiVector (device-resident column-major n x k
// block with an active-column mask) and the interpreter entries that make
// it a BLOPEX backend.  Replaces serial_Multi_Vector and the entries filled
// by SerialSetupInterpreter (blopex_serial_double/multivector/multi_vector.c,
// blopex_serial_double/pcg_multi/pcg_multi.c:14-242).
//
// Small matrices passed through the interpreter (MultiInnerProd,
// MultiVecMat, ...) are host arrays, as in the reference; the device solver
// in lobpcg_driver.c bypasses these entries and keeps its Gram matrices on
// the device.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

static size_t esize(int dtype) { return dtype == GPU_MV_FLOAT64 ? 8 : 4; }

static long pad_ld(long n) { return (n + 31) / 32 * 32; }

static gpu_MultiVector* mv_alloc(gpu_Context* ctx, long n, int k, int dtype)
{
  gpu_MultiVector* x = (gpu_MultiVector*)calloc(1, sizeof(gpu_MultiVector));
  if (!x) return NULL;
  x->size = n;
  x->ld = pad_ld(n);
  x->num_vectors = k;
  x->dtype = dtype;
  x->ctx = ctx;
  x->active = (BlopexInt*)malloc(sizeof(BlopexInt) * (k > 0 ? k : 1));
  x->active_dev = (BlopexInt*)gb_device_alloc(ctx, sizeof(BlopexInt) * (k > 0 ? k : 1));
  for (int i = 0; i < k; i++) x->active[i] = i;
  x->num_active = k;
  if (!x->active || !x->active_dev) {
    free(x->active);
    gb_device_free(x->active_dev);
    free(x);
    return NULL;
  }
  if (k > 0 && gb_memcpy_h2d(ctx, x->active_dev, x->active, sizeof(BlopexInt) * k)) {
    free(x->active);
    gb_device_free(x->active_dev);
    free(x);
    return NULL;
  }
  return x;
}

extern "C" gpu_MultiVector* gpu_MultiVectorCreate(gpu_Context* ctx, long n, BlopexInt k,
                                                  BlopexInt dtype)
{
  if (!ctx || n <= 0 || k < 0 || (dtype != GPU_MV_FLOAT64 && dtype != GPU_MV_FLOAT32)) {
    if (ctx) gb_fail(ctx, "gpu_MultiVectorCreate: bad arguments n=%ld k=%d dtype=%d", n, k, dtype);
    return NULL;
  }
  gpu_MultiVector* x = mv_alloc(ctx, n, k, dtype);
  if (!x) return NULL;
  size_t bytes = esize(dtype) * (size_t)x->ld * (size_t)(k > 0 ? k : 1);
  x->data = gb_device_alloc(ctx, bytes);
  if (!x->data) {
    free(x->active);
    gb_device_free(x->active_dev);
    free(x);
    return NULL;
  }
  // padding rows and fresh columns start at zero
  cudaMemsetAsync(x->data, 0, bytes, (cudaStream_t)ctx->stream);
  x->owns_data = 1;
  return x;
}

extern "C" gpu_MultiVector* gpu_MultiVectorWrapDevice(gpu_Context* ctx, void* data, long n, long ld,
                                                      BlopexInt k, BlopexInt dtype)
{
  if (!ctx || !data || n <= 0 || ld < n || k < 0) {
    if (ctx) gb_fail(ctx, "gpu_MultiVectorWrapDevice: bad arguments");
    return NULL;
  }
  gpu_MultiVector* x = mv_alloc(ctx, n, k, dtype);
  if (!x) return NULL;
  x->ld = ld;
  x->data = data;
  x->owns_data = 0;
  return x;
}

extern "C" void gpu_MultiVectorDestroy(gpu_MultiVector* x)
{
  if (!x) return;
  if (x->owns_data == 2 && x->data) {
    // internal block: its storage goes back to the context's pool
    gb_pool_put(x->ctx, x->data,
                esize(x->dtype) * (size_t)x->ld * (size_t)(x->num_vectors > 0 ? x->num_vectors : 1));
  } else if (x->owns_data && x->data) {
    cudaStreamSynchronize((cudaStream_t)x->ctx->stream);
    gb_device_free(x->data);
  }
  gb_device_free(x->active_dev);
  free(x->active);
  free(x);
}

// the solver's internal blocks: storage from the context's pool (no
// cudaMalloc / cudaFree per solve for repeated solves of one shape)
extern "C" gpu_MultiVector* gb_mv_create_like(const gpu_MultiVector* x, int dtype)
{
  gpu_Context* ctx = x->ctx;
  const int k = x->num_vectors;
  gpu_MultiVector* y = mv_alloc(ctx, x->size, k, dtype);
  if (!y) return NULL;
  const size_t bytes = esize(dtype) * (size_t)y->ld * (size_t)(k > 0 ? k : 1);
  y->data = gb_pool_get(ctx, bytes);
  if (!y->data) {
    free(y->active);
    gb_device_free(y->active_dev);
    free(y);
    return NULL;
  }
  cudaMemsetAsync(y->data, 0, bytes, (cudaStream_t)ctx->stream);
  y->owns_data = 2;
  return y;
}

extern "C" int gb_mv_fill_cols(const gpu_MultiVector* x, blk_cols* t, int offset)
{
  const char* base = (const char*)x->data;
  const size_t stride = esize(x->dtype) * (size_t)x->ld;
  int n = x->num_active;
  if (offset + n > BLK_MAXCOLS) n = BLK_MAXCOLS - offset;  // callers check the width first
  for (int c = 0; c < n; c++) t->col[offset + c] = base + stride * x->active[c];
  return offset + n;
}

extern "C" void gb_mv_set_mask_host(gpu_MultiVector* x, const BlopexInt* mask)
{
  x->num_active = 0;
  for (int i = 0; i < x->num_vectors; i++)
    if (mask == NULL || mask[i]) x->active[x->num_active++] = i;
}

extern "C" int gb_mv_sync_mask(gpu_MultiVector* x)
{
  if (x->num_active == 0) return 0;
  return gb_memcpy_h2d(x->ctx, x->active_dev, x->active, sizeof(BlopexInt) * x->num_active);
}

static int host_to_dev(gpu_MultiVector* x, const double* host, long ldh)
{
  gpu_Context* ctx = x->ctx;
  const int k = x->num_vectors;
  if (k == 0) return 0;
  if (x->dtype == GPU_MV_FLOAT64) {
    if (gb_cuda_check(ctx, (int)cudaMemcpy2DAsync(x->data, sizeof(double) * x->ld, host,
                                                  sizeof(double) * ldh, sizeof(double) * x->size,
                                                  k, cudaMemcpyHostToDevice,
                                                  (cudaStream_t)ctx->stream),
                      "FromHost"))
      return -1;
    return gb_sync(ctx);
  }
  // FP32 storage: convert on the host column by column
  float* tmp = (float*)malloc(sizeof(float) * x->size);
  if (!tmp) return gb_fail(ctx, "FromHost: host allocation failed");
  int rc = 0;
  for (int c = 0; c < k && !rc; c++) {
    for (long r = 0; r < x->size; r++) tmp[r] = (float)host[(size_t)c * ldh + r];
    rc = gb_memcpy_h2d(ctx, (float*)x->data + (size_t)c * x->ld, tmp, sizeof(float) * x->size);
  }
  free(tmp);
  return rc;
}

extern "C" int gpu_MultiVectorFromHost(gpu_MultiVector* x, const double* host, long ldh)
{
  if (ldh < x->size) return gb_fail(x->ctx, "FromHost: ldh < n");
  return host_to_dev(x, host, ldh);
}

extern "C" int gpu_MultiVectorToHost(gpu_MultiVector* x, double* host, long ldh)
{
  gpu_Context* ctx = x->ctx;
  if (ldh < x->size) return gb_fail(ctx, "ToHost: ldh < n");
  const int k = x->num_vectors;
  if (k == 0) return 0;
  if (x->dtype == GPU_MV_FLOAT64) {
    if (gb_cuda_check(ctx, (int)cudaMemcpy2DAsync(host, sizeof(double) * ldh, x->data,
                                                  sizeof(double) * x->ld, sizeof(double) * x->size,
                                                  k, cudaMemcpyDeviceToHost,
                                                  (cudaStream_t)ctx->stream),
                      "ToHost"))
      return -1;
    return gb_sync(ctx);
  }
  float* tmp = (float*)malloc(sizeof(float) * x->size);
  if (!tmp) return gb_fail(ctx, "ToHost: host allocation failed");
  int rc = 0;
  for (int c = 0; c < k && !rc; c++) {
    rc = gb_memcpy_d2h(ctx, tmp, (float*)x->data + (size_t)c * x->ld, sizeof(float) * x->size);
    for (long r = 0; r < x->size && !rc; r++) host[(size_t)c * ldh + r] = tmp[r];
  }
  free(tmp);
  return rc;
}

extern "C" int gpu_MultiVectorCopy(gpu_MultiVector* src, gpu_MultiVector* dst)
{
  if (src->size != dst->size || src->num_vectors != dst->num_vectors)
    return gb_fail(src->ctx, "gpu_MultiVectorCopy: shapes differ");
  blk_cols a, b;
  const size_t es = esize(src->dtype), ed = esize(dst->dtype);
  for (int c0 = 0; c0 < src->num_vectors; c0 += BLK_MAXCOLS) {
    int w = src->num_vectors - c0 < BLK_MAXCOLS ? src->num_vectors - c0 : BLK_MAXCOLS;
    for (int c = 0; c < w; c++) {
      a.col[c] = (const char*)src->data + es * (size_t)src->ld * (c0 + c);
      b.col[c] = (const char*)dst->data + ed * (size_t)dst->ld * (c0 + c);
    }
    if (gb_convert(src->ctx, src->size, src->dtype, &a, dst->dtype, &b, w)) return -1;
  }
  return 0;
}

extern "C" int gpu_MultiVectorSetRandomValues(gpu_MultiVector* x, BlopexInt seed)
{
  if (x->num_active > BLK_MAXCOLS)
    return gb_fail(x->ctx, "SetRandomValues: %d active columns exceed %d", x->num_active,
                   BLK_MAXCOLS);
  return gb_drand48_fill(x->ctx, x->dtype, x->data, x->size, x->ld, x->active, x->num_active,
                         (unsigned int)seed);
}

// ---------------------------------------------------------------------------
// interpreter entries (same contracts as pcg_multi.c:14-163)
// ---------------------------------------------------------------------------
static gpu_MultiVector* MV(void* p) { return (gpu_MultiVector*)p; }

// the block kernels address at most BLK_MAXCOLS columns per operand
static int too_wide(gpu_MultiVector* x)
{
  if (x->num_active <= BLK_MAXCOLS) return 0;
  gb_fail(x->ctx, "%d active columns exceed the supported %d", x->num_active, BLK_MAXCOLS);
  return 1;
}

static void* gi_CopyCreate(void* src_, BlopexInt copyValues)
{
  gpu_MultiVector* src = MV(src_);
  gpu_MultiVector* y = gpu_MultiVectorCreate(src->ctx, src->size, src->num_vectors, src->dtype);
  if (y && copyValues)
    gb_memcpy_d2d(src->ctx, y->data, src->data,
                  esize(src->dtype) * (size_t)src->ld * (size_t)src->num_vectors);
  return y;
}

static void gi_Destroy(void* x) { gpu_MultiVectorDestroy(MV(x)); }

static BlopexInt gi_Width(void* x) { return MV(x)->num_vectors; }

static BlopexInt gi_Height(void* x) { return (BlopexInt)MV(x)->size; }

static void gi_SetMask(void* x_, BlopexInt* mask)
{
  gpu_MultiVector* x = MV(x_);
  gb_mv_set_mask_host(x, mask);
  gb_mv_sync_mask(x);
}

static void gi_Copy(void* x_, void* y_)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  if (x->num_active != y->num_active) {
    gb_fail(x->ctx, "CopyMultiVector: active widths differ (%d vs %d)", x->num_active,
            y->num_active);
    return;
  }
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  gb_convert(x->ctx, x->size, x->dtype, &a, y->dtype, &b, x->num_active);
}

static void gi_Clear(void* x_)
{
  gpu_MultiVector* x = MV(x_);
  if (too_wide(x)) return;
  blk_cols a;
  gb_mv_fill_cols(x, &a, 0);
  gb_axpby(x->ctx, x->dtype, x->size, 0.0, &a, 0.0, &a, x->num_active);
}

static void gi_SetRandom(void* x, BlopexInt seed) { gpu_MultiVectorSetRandomValues(MV(x), seed); }

static void gi_InnerProd(void* x_, void* y_, BlopexInt gh, BlopexInt h, BlopexInt w, void* v)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  gpu_Context* ctx = x->ctx;
  if (x->num_active != h || y->num_active != w) {
    gb_fail(ctx, "MultiInnerProd: shape mismatch");
    return;
  }
  double* g = (double*)gb_device_alloc(ctx, sizeof(double) * (size_t)(h > 0 ? h : 1) * (w > 0 ? w : 1));
  if (!g) return;
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  if (gb_gram(ctx, x->dtype, x->size, &a, h, &b, w, g, h) == 0) {
    double* tmp = (double*)malloc(sizeof(double) * (size_t)h * w);
    if (gb_memcpy_d2h(ctx, tmp, g, sizeof(double) * (size_t)h * w) == 0)
      for (int j = 0; j < w; j++)
        for (int i = 0; i < h; i++) ((double*)v)[i + (size_t)j * gh] = tmp[i + (size_t)j * h];
    free(tmp);
  }
  gb_device_free(g);
}

static void gi_InnerProdDiag(void* x_, void* y_, BlopexInt* mask, BlopexInt n, void* diag)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  gpu_Context* ctx = x->ctx;
  int idx[BLK_MAXCOLS], na = 0;
  for (int i = 0; i < n; i++)
    if (mask == NULL || mask[i]) idx[na++] = i;
  if (na != x->num_active || na != y->num_active) {
    gb_fail(ctx, "MultiInnerProdDiag: mask does not match the active columns");
    return;
  }
  double* d = (double*)gb_device_alloc(ctx, sizeof(double) * (n > 0 ? n : 1));
  if (!d) return;
  double* host = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
  memcpy(host, diag, sizeof(double) * n);
  gb_memcpy_h2d(ctx, d, host, sizeof(double) * n);
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  if (gb_dot_cols(ctx, x->dtype, x->size, &a, &b, na, d, idx) == 0)
    gb_memcpy_d2h(ctx, diag, d, sizeof(double) * n);
  free(host);
  gb_device_free(d);
}

static void vecmat(void* x_, BlopexInt gh, BlopexInt h, BlopexInt w, void* v, void* y_, int add)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  gpu_Context* ctx = x->ctx;
  if (x->num_active != h || y->num_active != w) {
    gb_fail(ctx, "MultiVecMat: shape mismatch");
    return;
  }
  double* c = (double*)gb_device_alloc(ctx, sizeof(double) * (size_t)(h > 0 ? h : 1) * (w > 0 ? w : 1));
  if (!c) return;
  double* tmp = (double*)malloc(sizeof(double) * (size_t)h * w);
  for (int j = 0; j < w; j++)
    for (int i = 0; i < h; i++) tmp[i + (size_t)j * h] = ((double*)v)[i + (size_t)j * gh];
  gb_memcpy_h2d(ctx, c, tmp, sizeof(double) * (size_t)h * w);
  free(tmp);
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  gb_bymat(ctx, x->dtype, x->size, &a, h, c, h, &b, w, add ? &b : NULL);
  gb_sync(ctx);
  gb_device_free(c);
}

static void gi_VecMat(void* x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v, void* y)
{
  vecmat(x, gh, h, w, v, y, 0);
}

static void gi_Xapy(void* x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v, void* y)
{
  vecmat(x, gh, h, w, v, y, 1);
}

static void gi_VecMatDiag(void* x_, BlopexInt* mask, BlopexInt n, void* diag, void* y_)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  gpu_Context* ctx = x->ctx;
  int idx[BLK_MAXCOLS], na = 0;
  for (int i = 0; i < n; i++)
    if (mask == NULL || mask[i]) idx[na++] = i;
  if (na != x->num_active || na != y->num_active) {
    gb_fail(ctx, "MultiVecMatDiag: mask does not match the active columns");
    return;
  }
  double* d = (double*)gb_device_alloc(ctx, sizeof(double) * (n > 0 ? n : 1));
  if (!d) return;
  gb_memcpy_h2d(ctx, d, diag, sizeof(double) * n);
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  gb_scale_cols(ctx, x->dtype, x->size, &a, d, idx, &b, na);
  gb_sync(ctx);
  gb_device_free(d);
}

static void gi_Axpy(double alpha, void* x_, void* y_)
{
  gpu_MultiVector *x = MV(x_), *y = MV(y_);
  if (too_wide(x) || too_wide(y)) return;
  if (x->num_active != y->num_active) {
    gb_fail(x->ctx, "MultiAxpy: active widths differ");
    return;
  }
  blk_cols a, b;
  gb_mv_fill_cols(x, &a, 0);
  gb_mv_fill_cols(y, &b, 0);
  gb_axpby(x->ctx, x->dtype, x->size, alpha, &a, 1.0, &b, x->num_active);
}

static void gi_Print(void* x_, char* tag, BlopexInt limit)
{
  gpu_MultiVector* x = MV(x_);
  printf("======= %s =========\n", tag);
  printf("size %ld\n", x->size);
  printf("owns data %d\n", (int)x->owns_data);
  printf("num vectors %d\n", (int)x->num_vectors);
  printf("num active vectors  %d\n", (int)x->num_active);
  long rows = x->size;
  int cols = x->num_active;
  if (limit != 0) {
    if (rows > limit) rows = limit;
    if (cols > limit) cols = limit;
  }
  double* col = (double*)malloc(sizeof(double) * x->size);
  for (int c = 0; c < cols; c++) {
    if (x->dtype == GPU_MV_FLOAT64) {
      gb_memcpy_d2h(x->ctx, col, (double*)x->data + (size_t)x->active[c] * x->ld,
                    sizeof(double) * rows);
    } else {
      float* f = (float*)malloc(sizeof(float) * rows);
      gb_memcpy_d2h(x->ctx, f, (float*)x->data + (size_t)x->active[c] * x->ld, sizeof(float) * rows);
      for (long r = 0; r < rows; r++) col[r] = f[r];
      free(f);
    }
    for (long r = 0; r < rows; r++) printf("%ld %d  %22.16e  \n", r, c, col[r]);
  }
  free(col);
}

static void gi_Eval(void (*f)(void*, void*, void*), void* par, void* x, void* y) { f(par, x, y); }

extern "C" BlopexInt GpuSetupInterpreter(mv_InterfaceInterpreter* i)
{
  memset(i, 0, sizeof(*i));
  i->CopyCreateMultiVector = gi_CopyCreate;
  i->DestroyMultiVector = gi_Destroy;
  i->Width = gi_Width;
  i->Height = gi_Height;
  i->SetMask = gi_SetMask;
  i->CopyMultiVector = gi_Copy;
  i->ClearMultiVector = gi_Clear;
  i->SetRandomVectors = gi_SetRandom;
  i->MultiInnerProd = gi_InnerProd;
  i->MultiInnerProdDiag = gi_InnerProdDiag;
  i->MultiVecMat = gi_VecMat;
  i->MultiVecMatDiag = gi_VecMatDiag;
  i->MultiAxpy = gi_Axpy;
  i->MultiPrint = gi_Print;
  i->MultiXapy = gi_Xapy;
  i->Eval = gi_Eval;
  return 0;
}

extern "C" int gb_is_gpu_interpreter(const mv_InterfaceInterpreter* ii)
{
  return ii && ii->MultiInnerProd == gi_InnerProd && ii->MultiVecMat == gi_VecMat;
}
