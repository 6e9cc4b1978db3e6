// lp_common.cuh — device primitives shared by the stages: block/warp scans, device-wide
// exclusive scan, bitonic sorts in shared memory, bounded-wait helpers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lp_internal.cuh"

namespace lpg
{
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems; // 2048 elements per block

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane_id() >= static_cast<uint32_t>(o))
            v += t;
    }
    return v;
}

// ---- TMA bulk copies (global -> shared) completing on an mbarrier ------------------------------
// cp.async.bulk moves a contiguous range (16-byte aligned, size a multiple of 16) through the
// tensor memory accelerator; the issuing thread announces the byte count on the mbarrier, and
// the barrier's phase flips when that many bytes have landed.
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
// Waits until the barrier has completed the phase with the given parity; gives up after
// `limit` polls and returns false (the caller reports it and stops using the buffer).
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; ++i)
    {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(bar)), "r"(parity)
            : "memory");
        if (done)
            return true;
    }
    return false;
}

// Warp-aggregated counter increment: every valid lane adds 1 to counters[key] and receives the
// counter's old value plus its rank among the valid lanes with the same key, as if the lanes'
// atomicAdds had run in lane order. One atomic per distinct key of the warp (consecutive points
// of a cluster or cell share a counter, so same-address atomics drop by up to 32x). All 32 lanes
// must call it; invalid lanes take no part and receive 0.
__device__ __forceinline__ uint32_t warp_aggregated_inc(uint32_t* counters, uint32_t key, bool valid)
{
    const uint32_t lane = lane_id();
    const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
    const uint32_t peers = __match_any_sync(0xffffffffu, valid ? key : 0xffffffffu) & vmask;
    const uint32_t leader = peers ? static_cast<uint32_t>(__ffs(peers) - 1) : lane;
    uint32_t old = 0u;
    if (valid && lane == leader)
        old = atomicAdd(&counters[key], static_cast<uint32_t>(__popc(peers)));
    old = __shfl_sync(0xffffffffu, old, static_cast<int>(leader));
    return valid ? old + static_cast<uint32_t>(__popc(peers & ((1u << lane) - 1u))) : 0u;
}

__device__ __forceinline__ uint32_t warp_sum(uint32_t v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Exclusive scan across the block (blockDim.x == kScanThreads); returns the exclusive prefix of
// v and writes the block total to *total. smem: kScanThreads / 32 + 1 words.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* smem, uint32_t* total)
{
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t nw = blockDim.x >> 5;
    const uint32_t incl = warp_incl_scan(v);
    if (lane == 31)
        smem[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        const uint32_t w = (lane < nw) ? smem[lane] : 0u;
        const uint32_t wi = warp_incl_scan(w);
        if (lane < nw)
            smem[lane] = wi - w;
        if (lane == nw - 1)
            smem[32] = wi;
    }
    __syncthreads();
    const uint32_t res = smem[warp] + incl - v;
    *total = smem[32];
    __syncthreads();
    return res;
}


// Bitonic sort of `n` (power of two) keys in shared memory by the whole block.
template <typename T, typename Less>
__device__ void block_bitonic_sort(T* s, uint32_t n, Less less)
{
    for (uint32_t k = 2; k <= n; k <<= 1)
    {
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            for (uint32_t i = threadIdx.x; i < n; i += blockDim.x)
            {
                const uint32_t ixj = i ^ j;
                if (ixj > i)
                {
                    const bool up = ((i & k) == 0);
                    T a = s[i], b = s[ixj];
                    const bool swap = up ? less(b, a) : less(a, b);
                    if (swap)
                    {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Bitonic sort of `n` (power of two) keys in shared memory by one full warp.
template <typename T, typename Less>
__device__ void warp_bitonic_smem(T* s, uint32_t n, Less less)
{
    for (uint32_t k = 2; k <= n; k <<= 1)
    {
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            for (uint32_t i = lane_id(); i < n; i += 32)
            {
                const uint32_t ixj = i ^ j;
                if (ixj > i)
                {
                    const bool up = ((i & k) == 0);
                    T a = s[i], b = s[ixj];
                    if (up ? less(b, a) : less(a, b))
                    {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncwarp();
        }
    }
}

// Bitonic sort of 32 values held one per lane (ascending by lane).
template <typename T, typename Less>
__device__ __forceinline__ T warp_bitonic_sort(T v, Less less)
{
    const uint32_t lane = lane_id();
#pragma unroll
    for (uint32_t k = 2; k <= 32; k <<= 1)
    {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            const T o = __shfl_xor_sync(0xffffffffu, v, j);
            const bool up = ((lane & k) == 0);
            const bool lower = ((lane & j) == 0);
            // lower lane keeps min when ascending
            const bool take_o = (lower == up) ? less(o, v) : less(v, o);
            if (take_o)
                v = o;
        }
    }
    return v;
}

__host__ __device__ inline uint32_t next_pow2(uint32_t v)
{
    v--;
    v |= v >> 1;
    v |= v >> 2;
    v |= v >> 4;
    v |= v >> 8;
    v |= v >> 16;
    return v + 1;
}

__host__ __device__ inline uint32_t div_up(uint32_t a, uint32_t b)
{
    return (a + b - 1) / b;
}
} // namespace lpg
