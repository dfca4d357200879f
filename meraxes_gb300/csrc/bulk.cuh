// Bulk asynchronous copies global -> shared memory (cp.async.bulk) with
// completion on an mbarrier, and bounded waits on the barrier.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace mx {
namespace bulk {

constexpr unsigned ERR_PIPELINE_TIMEOUT = 2u;
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;  // 2 s
constexpr long long WAIT_LIMIT_ITERS = 1LL << 26;

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arms the barrier for `bytes` of bulk copies (one arrival).  Orders this
// thread's earlier generic-proxy shared-memory accesses before the copies.
__device__ __forceinline__ void mbar_arm(uint64_t* bar, unsigned bytes)
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// One bulk copy global -> shared completing on `bar`.  dst, src and bytes are
// multiples of 16.
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
  asm volatile(
    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
    "l"(src), "r"(bytes), "r"(smem_addr(bar))
    : "memory");
}

// Opaque copy of a CUtensorMap (128 bytes, 64-byte aligned), so that kernel
// headers need not include the driver API.  Passed to kernels as a
// __grid_constant__ parameter.
struct alignas(64) TensorMap
{
  unsigned long long v[16];
};

// One tiled tensor copy of the box at coordinates (x, y) of a 2-D tensor map
// into shared memory (128-byte aligned), completing on `bar`.  x times the
// element size is a multiple of 16 bytes.
__device__ __forceinline__ void bulk_tensor_2d(void* dst, const TensorMap* map, int x, int y, uint64_t* bar)
{
  asm volatile(
    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
      smem_addr(dst)),
    "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
    : "memory");
}

// Arms the barrier for `bytes` and issues one bulk copy of that size.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar)
{
  mbar_arm(bar, bytes);
  bulk_copy(dst, src, bytes, bar);
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity)
{
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_addr(bar)), "r"(parity)
    : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns()
{
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Polls a consumer's wait may take before it gives up (at most
// WAIT_LIMIT_ITERS, and never longer than WAIT_LIMIT_NS).  One copy per
// translation unit; set_consumer_wait_polls() sets this unit's copy.  A
// context sets it when it is created: the default, or a lower value that a
// test of the give-up path asks for (MX_WAIT_POLL_LIMIT).
static __device__ long long consumer_wait_polls = WAIT_LIMIT_ITERS;

static inline cudaError_t set_consumer_wait_polls(long long polls)
{
  return cudaMemcpyToSymbol(consumer_wait_polls, &polls, sizeof(polls));
}

// Non-blocking test of the phase (mbarrier.test_wait); mbar_test's try_wait
// may suspend the thread for a while before it returns false.
__device__ __forceinline__ bool mbar_test_now(uint64_t* bar, unsigned parity)
{
  uint32_t ok;
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
    "selp.u32 %0, 1, 0, p;\n\t}"
    : "=r"(ok)
    : "r"(smem_addr(bar)), "r"(parity)
    : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_polls(uint64_t* bar, unsigned parity, long long polls)
{
  if (polls < WAIT_LIMIT_ITERS) {
    // a lowered limit (a test of the give-up path): polls that do not wait
    for (long long it = 0; it < polls; it++)
      if (mbar_test_now(bar, parity))
        return true;
    return false;
  }
  if (mbar_test(bar, parity))
    return true;
  const unsigned long long t0 = global_ns();
  for (long long it = 1; it < polls; it++) {
    if (mbar_test(bar, parity))
      return true;
    if ((it & 255) == 0 && global_ns() - t0 > WAIT_LIMIT_NS)
      return false;
  }
  return false;
}

// A consumer's wait for phase `parity` of the barrier; false when it gives
// up (consumer_wait_polls polls, or about WAIT_LIMIT_NS).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity)
{
  return mbar_wait_polls(bar, parity, consumer_wait_polls);
}

// The wait of a block that gave up, for its own copies still in flight
// before it exits: always the full limit, whatever the consumers' limit.
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, unsigned parity)
{
  return mbar_wait_polls(bar, parity, WAIT_LIMIT_ITERS);
}

}  // namespace bulk
}  // namespace mx
