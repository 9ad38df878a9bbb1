// tma.cuh - the bulk-tensor (TMA) copies and mbarrier waits of the
// persistent FP32 step kernel, as inline PTX for sm_103a.
//
// Loads: cp.async.bulk.tensor.3d (x = cells along z, y = rows along r,
// z = the four state planes) into shared memory, completion signalled on an
// mbarrier with an expected byte count.  Stores: the updated tile from
// shared memory back to the state planes through a bulk group.  Every wait
// is bounded: after its limit of failed polls the caller gets `false` and
// must report the failure instead of waiting on.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ast {
namespace tma {

constexpr int kWaitLimit = 1 << 21;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// orders this thread's shared-memory writes (generic proxy) before later
// accesses by the bulk-copy engine (async proxy), and makes an mbarrier's
// initialisation visible to it
__device__ __forceinline__ void fence_async_shared()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// arms the barrier for `bytes` of incoming data (one arrival)
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// waits for the completion of phase `parity` of the barrier; false after
// `limit` polls.  The default limit polls with try_wait, which may suspend
// the thread between polls (about a second in all); a shorter limit (a
// configured copy_wait_polls, the failure tests' setting) polls with the
// non-blocking test_wait, so that it runs out within microseconds
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kWaitLimit)
{
    const uint32_t a = smem_addr(bar);
    if (limit < kWaitLimit) {
        for (int i = 0; i < limit; i++) {
            uint32_t done;
            asm volatile(
                "{\n"
                ".reg .pred p;\n"
                "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                "selp.u32 %0, 1, 0, p;\n"
                "}\n"
                : "=r"(done)
                : "r"(a), "r"(parity)
                : "memory");
            if (done) return true;
        }
        return false;
    }
    for (int i = 0; i < kWaitLimit; i++) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.u32 %0, 1, 0, p;\n"
            "}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// box of the 3-D tensor map at (x, y, z) into shared memory, completing on bar
__device__ __forceinline__ void load_3d(const CUtensorMap* map, void* dst, uint64_t* bar, int x, int y, int z)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}

// `bytes` contiguous bytes from global memory into shared memory,
// completing on bar (both addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void load_bulk(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

// asynchronous copies of 8 / 16 bytes from global to shared memory with no
// register staging (cp.async, completed by async_wait_all in this thread)
__device__ __forceinline__ void async_copy8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void async_copy16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// shared-memory box to the tensor at (x, y, z); parts outside the tensor
// are not written
__device__ __forceinline__ void store_3d(const CUtensorMap* map, const void* src, int x, int y, int z)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%1, %2, %3}], [%4];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(src))
                 : "memory");
}

__device__ __forceinline__ void store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// the committed stores have read their shared-memory source
__device__ __forceinline__ void store_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// the committed stores are complete
__device__ __forceinline__ void store_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

}  // namespace tma
}  // namespace ast
