// tma.cuh -- Tensor Memory Accelerator copies, mbarriers and bounded waits (sm_90+ PTX, used on sm_103a).
//
// A tile copy is one cp.async.bulk.tensor instruction issued by one thread:
// global -> shared completes on an mbarrier (transaction bytes), shared ->
// global completes through a bulk group.  Every wait is bounded by the
// global nanosecond timer: a wait that runs out sets a bit in the launch's
// device status word, which the host reads back as GOPF_ERR_TIMEOUT.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gopf {

// DS_TMA_TIMEOUT: a tile copy's wait ran out; DS_DEP_TIMEOUT: a persistent kernel's wait for the
// items an item depends on ran out
enum DeviceStatusBits : unsigned { DS_TMA_TIMEOUT = 1u, DS_DEP_TIMEOUT = 2u };

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the initialised barrier visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

// order this thread's shared-memory writes before later async-proxy reads (TMA stores)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

// Wait for phase `parity` of the barrier for at most `limit_ns`; false on timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, unsigned long long limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

// Wait for a TMA load's barrier.  On timeout: flag the status word, wait once
// more (bounded by the built-in 2 s) for the copy still in flight, and report
// failure so the caller returns without touching the tile.  The first wait's
// limit is the unsigned long long at status + 2 when it is non-zero (a context
// option, GOPF_OPT_WAIT_LIMIT_NS), else 2 s; the second wait never shortens, so
// a block leaves only after its copy has landed.
__device__ __forceinline__ bool tma_wait_or_flag(uint64_t *bar, uint32_t parity, unsigned *status)
{
    const unsigned long long lim = 2000000000ull; // 2 s: orders of magnitude above a 32 KB copy
    unsigned long long first = lim;
    if (status) {
        const unsigned long long l = *reinterpret_cast<const volatile unsigned long long *>(status + 2);
        if (l) first = l;
    }
    if (mbar_wait_bounded(bar, parity, first)) return true;
    if (status) atomicOr(status, (unsigned)DS_TMA_TIMEOUT);
    mbar_wait_bounded(bar, parity, lim);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, int x, int y, const void *src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, int x, int y, int z, const void *src)
{
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(z), "r"(smem_u32(src))
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// the shared-memory sources of all committed bulk stores have been read
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Host: encode a tiled tensor map of 8-byte elements (float2), rank 2 or 3.
// dims[0] is contiguous; strides_bytes[i] is the byte stride of dims[i+1].
// Returns false when the driver entry point is missing or rejects the map.
bool encode_map_8b(CUtensorMap *map, const void *base, int rank, const unsigned long long *dims,
                   const unsigned long long *strides_bytes, const unsigned *box);

} // namespace gopf
