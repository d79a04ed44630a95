// context.cu -- device context: stream, scratch memory, options, errors.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "internal.h"

static long long g_launches = 0;

static const char* k_names[GB_K_COUNT] = {"gram", "xc_update", "spmm_csr", "stencil7",
                                          "stencil5", "stencil27", "diag_scale", "residual",
                                          "blas1", "cholqr", "sygv", "small_dense", "tc_gram",
                                          "tc_xc_update", "sygv_fp64_gate", "rr_chol64",
                                          "rr_trsm64", "rr_jacobi32", "rr_gemm64", "rr_refine",
                                          "rr_tridiag", "rr_tridiag_eig", "gram_fp32",
                                          "xc_update_fp32", "spmm_csr_fp32", "stencil7_fp32",
                                          "stencil5_fp32", "stencil27_fp32", "diag_scale_fp32",
                                          "oz_xc_update", "oz_gram"};


extern "C" void gb_count_launch(long long n) { __atomic_fetch_add(&g_launches, n, __ATOMIC_RELAXED); }

extern "C" long long gpu_KernelLaunchCount(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

extern "C" double gb_now(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

extern "C" int gb_fail(gpu_Context* ctx, const char* fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  if (ctx) {
    vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
  } else {
    vfprintf(stderr, fmt, ap);
    fputc('\n', stderr);
  }
  va_end(ap);
  return -1;
}

extern "C" int gb_cuda_check(gpu_Context* ctx, int status, const char* what)
{
  if (status == cudaSuccess) return 0;
  return gb_fail(ctx, "CUDA error in %s: %s", what, cudaGetErrorString((cudaError_t)status));
}

static void default_options(lobpcg_gpu_options* o)
{
  memset(o, 0, sizeof(*o));
  o->precision = LOBPCG_GPU_FP64;
  o->compensated_below = 1e-6;
  o->fp64_below = 0.0;
  o->accum64 = 0;
  o->fp32_accurate_op = 0;
  o->recompute_ap = 1;
  o->fp32_precond = 0;
  o->explicit_pivot_below = 1e-6;
  o->fp32_stall = 20;
  o->tensor_cores = 1;
  o->split_products = 1;
}

extern "C" gpu_Context* gpu_ContextCreate(int device, void* stream)
{
  gpu_Context* ctx = (gpu_Context*)calloc(1, sizeof(gpu_Context));
  if (!ctx) return NULL;
  if (device < 0) {
    if (cudaGetDevice(&device) != cudaSuccess) {
      free(ctx);
      return NULL;
    }
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    free(ctx);
    return NULL;
  }
  ctx->device = device;
  default_options(&ctx->opt);
  if (stream) {
    ctx->stream = stream;
  } else {
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      free(ctx);
      return NULL;
    }
    ctx->stream = (void*)s;
    ctx->owns_stream = 1;
  }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (ctx->num_sms <= 0) ctx->num_sms = 152;
  for (int c = 0; c < GB_K_COUNT; c++) strncpy(ctx->prof[c].name, k_names[c], sizeof(ctx->prof[c].name) - 1);
  if (cudaMalloc((void**)&ctx->dcount, 8 * sizeof(int)) != cudaSuccess ||
      cudaMemsetAsync(ctx->dcount, 0, 8 * sizeof(int), (cudaStream_t)ctx->stream) != cudaSuccess) {
    if (ctx->owns_stream) cudaStreamDestroy((cudaStream_t)ctx->stream);
    free(ctx);
    return NULL;
  }
  return ctx;
}

extern "C" void gb_prof_begin(gpu_Context* ctx, gb_prof_rec* rec, int cls)
{
  rec->start = rec->stop = NULL;
  rec->cls = cls;
  if (!ctx->profile) return;
  cudaEvent_t e[2];
  for (int i = 0; i < 2; i++) {
    if (ctx->prof_npool > 0)
      e[i] = (cudaEvent_t)ctx->prof_pool[--ctx->prof_npool];
    else if (cudaEventCreate(&e[i]) != cudaSuccess)
      return;
  }
  rec->start = (void*)e[0];
  rec->stop = (void*)e[1];
  cudaEventRecord(e[0], (cudaStream_t)ctx->stream);
}

extern "C" void gb_prof_end(gpu_Context* ctx, gb_prof_rec* rec, double bytes, double flops)
{
  if (!ctx->profile || !rec->start) return;
  cudaEventRecord((cudaEvent_t)rec->stop, (cudaStream_t)ctx->stream);
  rec->bytes = bytes;
  rec->flops = flops;
  if (ctx->prof_npending == ctx->prof_cap) {
    int cap = ctx->prof_cap ? 2 * ctx->prof_cap : 1024;
    gb_prof_rec* p = (gb_prof_rec*)realloc(ctx->prof_pending, sizeof(gb_prof_rec) * cap);
    if (!p) return;
    ctx->prof_pending = p;
    ctx->prof_cap = cap;
  }
  ctx->prof_pending[ctx->prof_npending++] = *rec;
}

static void pool_put(gpu_Context* ctx, void* ev)
{
  if (ctx->prof_npool % 256 == 0) {
    void** p = (void**)realloc(ctx->prof_pool, sizeof(void*) * (ctx->prof_npool + 256));
    if (!p) {
      cudaEventDestroy((cudaEvent_t)ev);
      return;
    }
    ctx->prof_pool = p;
  }
  ctx->prof_pool[ctx->prof_npool++] = ev;
}

extern "C" void gb_prof_collect(gpu_Context* ctx)
{
  if (ctx->prof_npending == 0) return;
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  for (int i = 0; i < ctx->prof_npending; i++) {
    gb_prof_rec* r = &ctx->prof_pending[i];
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, (cudaEvent_t)r->start, (cudaEvent_t)r->stop) == cudaSuccess) {
      lobpcg_gpu_kernel_time* t = &ctx->prof[r->cls];
      t->launches++;
      t->ms += ms;
      t->bytes += r->bytes;
      t->flops += r->flops;
    }
    pool_put(ctx, r->start);
    pool_put(ctx, r->stop);
  }
  ctx->prof_npending = 0;
}

extern "C" int gpu_ContextSetProfiling(gpu_Context* ctx, int on)
{
  gb_prof_collect(ctx);
  ctx->profile = on ? 1 : 0;
  return 0;
}

extern "C" void gpu_ContextResetKernelTimes(gpu_Context* ctx)
{
  gb_prof_collect(ctx);
  memset(ctx->prof, 0, sizeof(ctx->prof));
  for (int c = 0; c < GB_K_COUNT; c++) strncpy(ctx->prof[c].name, k_names[c], sizeof(ctx->prof[c].name) - 1);
}

extern "C" int gpu_ContextKernelTimes(gpu_Context* ctx, lobpcg_gpu_kernel_time* out, int max)
{
  gb_prof_collect(ctx);
  int n = 0;
  for (int c = 0; c < GB_K_COUNT && n < max; c++)
    if (ctx->prof[c].launches > 0) out[n++] = ctx->prof[c];
  return n;
}

extern "C" void gpu_ContextDestroy(gpu_Context* ctx)
{
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  gb_prof_collect(ctx);
  for (int i = 0; i < ctx->prof_npool; i++) cudaEventDestroy((cudaEvent_t)ctx->prof_pool[i]);
  free(ctx->prof_pool);
  free(ctx->prof_pending);
  if (ctx->work) cudaFree(ctx->work);
  gpu_ContextTrim(ctx);
  if (ctx->dcount) cudaFree(ctx->dcount);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->owns_stream) cudaStreamDestroy((cudaStream_t)ctx->stream);
  free(ctx);
}

extern "C" void* gb_pool_get(gpu_Context* ctx, size_t bytes)
{
  for (int i = 0; i < ctx->pool_n; i++)
    if (ctx->pool_bytes[i] == bytes) {
      void* p = ctx->pool_ptr[i];
      ctx->pool_n--;
      ctx->pool_ptr[i] = ctx->pool_ptr[ctx->pool_n];
      ctx->pool_bytes[i] = ctx->pool_bytes[ctx->pool_n];
      return p;
    }
  return gb_device_alloc(ctx, bytes);
}

extern "C" void gb_pool_put(gpu_Context* ctx, void* p, size_t bytes)
{
  if (!p) return;
  if (ctx->pool_n < GB_POOL_MAX) {
    ctx->pool_ptr[ctx->pool_n] = p;
    ctx->pool_bytes[ctx->pool_n] = bytes;
    ctx->pool_n++;
    return;
  }
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  gb_device_free(p);
}

extern "C" void gpu_ContextTrim(gpu_Context* ctx)
{
  if (!ctx || ctx->pool_n == 0) return;
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  for (int i = 0; i < ctx->pool_n; i++) gb_device_free(ctx->pool_ptr[i]);
  ctx->pool_n = 0;
}

extern "C" void* gpu_ContextStream(gpu_Context* ctx) { return ctx ? ctx->stream : NULL; }

extern "C" int gpu_ContextSynchronize(gpu_Context* ctx)
{
  return gb_cuda_check(ctx, cudaStreamSynchronize((cudaStream_t)ctx->stream),
                       "cudaStreamSynchronize");
}

extern "C" void gpu_ContextGetOptions(gpu_Context* ctx, lobpcg_gpu_options* opt) { *opt = ctx->opt; }

extern "C" int gpu_ContextSetOptions(gpu_Context* ctx, const lobpcg_gpu_options* opt)
{
  if (opt->precision != LOBPCG_GPU_FP64 && opt->precision != LOBPCG_GPU_MIXED)
    return gb_fail(ctx, "unknown precision mode %d", opt->precision);
  if (opt->wait_polls < 0) return gb_fail(ctx, "wait_polls must be >= 0 (0 = default)");
  ctx->opt = *opt;
  return 0;
}

extern "C" void gpu_ContextGetStats(gpu_Context* ctx, lobpcg_gpu_stats* stats) { *stats = ctx->stats; }

extern "C" const char* gpu_ContextLastError(gpu_Context* ctx) { return ctx ? ctx->err : ""; }

extern "C" void* gb_workspace(gpu_Context* ctx, size_t bytes)
{
  if (bytes <= ctx->work_bytes) return ctx->work;
  // growing: the old scratch may still be read by queued kernels
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  if (ctx->work) cudaFree(ctx->work);
  ctx->work = NULL;
  ctx->work_bytes = 0;
  size_t want = bytes + bytes / 4 + 4096;
  if (cudaMalloc(&ctx->work, want) != cudaSuccess) {
    gb_fail(ctx, "cudaMalloc of %zu scratch bytes failed", want);
    return NULL;
  }
  ctx->work_bytes = want;
  return ctx->work;
}

extern "C" void* gb_pinned(gpu_Context* ctx, size_t bytes)
{
  if (bytes <= ctx->pinned_bytes) return ctx->pinned;
  cudaStreamSynchronize((cudaStream_t)ctx->stream);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  ctx->pinned = NULL;
  ctx->pinned_bytes = 0;
  size_t want = bytes < 65536 ? 65536 : bytes;
  if (cudaMallocHost(&ctx->pinned, want) != cudaSuccess) {
    gb_fail(ctx, "cudaMallocHost of %zu bytes failed", want);
    return NULL;
  }
  ctx->pinned_bytes = want;
  return ctx->pinned;
}

extern "C" int gb_memcpy_d2h(gpu_Context* ctx, void* dst, const void* src, size_t bytes)
{
  if (bytes == 0) return 0;
  cudaStream_t s = (cudaStream_t)ctx->stream;
  if (gb_cuda_check(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s), "d2h copy"))
    return -1;
  return gb_cuda_check(ctx, cudaStreamSynchronize(s), "d2h sync");
}

extern "C" int gb_memcpy_h2d(gpu_Context* ctx, void* dst, const void* src, size_t bytes)
{
  if (bytes == 0) return 0;
  cudaStream_t s = (cudaStream_t)ctx->stream;
  if (gb_cuda_check(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s), "h2d copy"))
    return -1;
  // the host buffer may be reused by the caller right away
  return gb_cuda_check(ctx, cudaStreamSynchronize(s), "h2d sync");
}

extern "C" int gb_memcpy_d2d(gpu_Context* ctx, void* dst, const void* src, size_t bytes)
{
  if (bytes == 0) return 0;
  return gb_cuda_check(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice,
                                            (cudaStream_t)ctx->stream), "d2d copy");
}

extern "C" int gb_sync(gpu_Context* ctx)
{
  return gb_cuda_check(ctx, cudaStreamSynchronize((cudaStream_t)ctx->stream), "sync");
}

extern "C" void* gb_device_alloc(gpu_Context* ctx, size_t bytes)
{
  void* p = NULL;
  if (bytes == 0) bytes = 256;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    gb_fail(ctx, "cudaMalloc of %zu bytes failed", bytes);
    return NULL;
  }
  return p;
}

extern "C" void gb_device_free(void* p)
{
  if (p) cudaFree(p);
}
