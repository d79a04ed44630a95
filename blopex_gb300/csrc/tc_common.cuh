// tc_common.cuh -- inline-PTX building blocks shared by the tcgen05
// kernels (tc_gram.cu, tc_xc.cu): shared-memory mbarriers with bounded waits,
// cp.async, the 128-byte-swizzled K-major shared-memory descriptor, the TF32
// instruction descriptor, tcgen05.mma / commit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define TC_WAIT_LIMIT (1L << 24)  // polls of one bounded mbarrier wait (default)

// The pipeline waits' poll limit, one copy per translation unit (no
// relocatable device code): tc_apply_wait_polls brings it in line with the
// launching context's option before each launch.  The drains (copies in
// flight, the issuer's final commit before TMEM is freed) always use
// TC_WAIT_LIMIT, so a short limit cannot let a CTA exit with work in flight.
static __constant__ long tc_wait_polls = TC_WAIT_LIMIT;
static long tc_wait_polls_host = TC_WAIT_LIMIT;  // the value last written to tc_wait_polls

static inline cudaError_t tc_apply_wait_polls(int polls, cudaStream_t stream)
{
  const long v = polls > 0 ? (long)polls : TC_WAIT_LIMIT;
  if (v == tc_wait_polls_host) return cudaSuccess;
  // a pageable source is staged before the call returns
  const cudaError_t e =
      cudaMemcpyToSymbolAsync(tc_wait_polls, &v, sizeof v, 0, cudaMemcpyHostToDevice, stream);
  if (e == cudaSuccess) tc_wait_polls_host = v;
  return e;
}

static __device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

// the first 1024-byte boundary at or after p in shared memory, by pointer
// arithmetic on p: the compiler then still sees a shared-memory pointer and
// emits shared loads and stores through it (a round trip through an integer
// makes every access generic, with the latency of a global access)
static __device__ __forceinline__ unsigned char* smem_align1024(unsigned char* p)
{
  return p + ((1024u - (smem_u32(p) & 1023u)) & 1023u);
}

static __device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

static __device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_u32(bar))
               : "memory");
}

static __device__ __forceinline__ bool mbar_try_wait(uint32_t addr, uint32_t parity)
{
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(done)
      : "r"(addr), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded pipeline wait for the phase with the given parity (tc_wait_polls
// polls); false on timeout or when another role has aborted
static __device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
  const uint32_t addr = smem_u32(bar);
  const long limit = tc_wait_polls;
  for (long i = 0; i < limit; i++) {
    if (mbar_try_wait(addr, parity)) return true;
    if (*abort_flag) return false;
  }
  return false;
}

// bounded drain: wait for work already in flight (copies landing in this
// CTA's shared memory, the MMAs before TMEM is freed); never aborted early
static __device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity)
{
  const uint32_t addr = smem_u32(bar);
  for (long i = 0; i < TC_WAIT_LIMIT; i++)
    if (mbar_try_wait(addr, parity)) return true;
  return false;
}

static __device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t bytes)
{
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(bytes)
               : "memory");
}

static __device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
static __device__ __forceinline__ void cp_async_wait()
{
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

static __device__ __forceinline__ void fence_proxy_async()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
static __device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr)
{
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
  d |= (uint64_t)1 << 16;                    // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024 >> 4) << 32;          // stride byte offset
  d |= (uint64_t)1 << 46;                    // descriptor version
  d |= (uint64_t)2 << 61;                    // SWIZZLE_128B
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, M x N
static __host__ __device__ constexpr uint32_t tf32_idesc(int M, int N)
{
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

static __device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

static __device__ __forceinline__ void mma_commit(uint64_t* bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}


static __device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
static __device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (lane i of the
// warp reads TMEM lane base + i); waits for the load
static __device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// x = hi + lo with hi representable in TF32 (low 13 mantissa bits cleared)
static __device__ __forceinline__ void tf32_split(float x, float& hi, float& lo)
{
  hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
  lo = x - hi;
}

// barrier among the `count` threads of the warps that use barrier `id` (> 0)
static __device__ __forceinline__ void named_bar(int id, int count)
{
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
