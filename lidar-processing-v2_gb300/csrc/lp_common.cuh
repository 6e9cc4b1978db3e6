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

// Block-wide version for counters many threads of a block may share even where the lanes of a
// warp do not (unordered input): the warps' groups of equal keys meet in a shared-memory table,
// and one global atomic per key and block reserves the block's total; a key the table cannot take
// (kBlockAggProbes probes) takes its own global atomic. Every thread of the block calls it (two
// barriers). Returns the thread's rank among its key's increments (unique, order unspecified).
constexpr uint32_t kBlockAggSlots = 512;
constexpr uint32_t kBlockAggProbes = 16;
static_assert(kBlockAggSlots == 512u, "the slot hash takes the top 9 bits");
struct BlockAgg
{
    uint32_t key[kBlockAggSlots];
    uint32_t cnt[kBlockAggSlots];
};

__device__ __forceinline__ uint32_t block_aggregated_inc(uint32_t* counters, uint32_t key, bool valid, BlockAgg& sh)
{
    constexpr uint32_t kFree = 0xffffffffu;
    const uint32_t lane = lane_id();
    for (uint32_t k = threadIdx.x; k < kBlockAggSlots; k += blockDim.x)
    {
        sh.key[k] = kFree;
        sh.cnt[k] = 0u;
    }
    const uint32_t vmask = __ballot_sync(0xffffffffu, valid);
    const uint32_t peers = __match_any_sync(0xffffffffu, valid ? key : kFree) & vmask;
    const uint32_t leader = peers ? static_cast<uint32_t>(__ffs(peers) - 1) : lane;
    __syncthreads();
    uint32_t slot = kFree, loc = 0u;
    if (valid && lane == leader)
    {
        uint32_t h = (key * 2654435761u) >> (32 - 9); // kBlockAggSlots = 2^9
        for (uint32_t probe = 0; probe < kBlockAggProbes; ++probe)
        {
            const uint32_t prev = atomicCAS(&sh.key[h], kFree, key);
            if (prev == kFree || prev == key)
            {
                slot = h;
                loc = atomicAdd(&sh.cnt[h], static_cast<uint32_t>(__popc(peers)));
                break;
            }
            h = (h + 1u) & (kBlockAggSlots - 1u);
        }
        if (slot == kFree)
            loc = atomicAdd(&counters[key], static_cast<uint32_t>(__popc(peers)));
    }
    __syncthreads();
    // the block's total per key: one global atomic each (the count is replaced by the key's base)
    for (uint32_t k = threadIdx.x; k < kBlockAggSlots; k += blockDim.x)
        if (sh.key[k] != kFree)
            sh.cnt[k] = atomicAdd(&counters[sh.key[k]], sh.cnt[k]);
    __syncthreads();
    uint32_t base = 0u;
    if (valid && lane == leader)
        base = (slot != kFree) ? sh.cnt[slot] + loc : loc;
    base = __shfl_sync(0xffffffffu, base, static_cast<int>(leader));
    return valid ? base + static_cast<uint32_t>(__popc(peers & ((1u << lane) - 1u))) : 0u;
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

// ---------------------------------------------------------------------------------------------
// Single-pass exclusive scan with decoupled look-back (Merrill & Garland, "Single-pass Parallel
// Prefix Scan with Decoupled Look-back", 2016). Tiles of kLbTile elements take dynamic tickets, so
// every tile a block waits for has already started (and waits only for earlier ones): each
// look-back ends. A tile publishes (flag, value) in one 64-bit word: flag 1 = the tile's own sum,
// flag 2 = the inclusive prefix through the tile. Waits are bounded anyway; running out sets
// ERR_INTERNAL in *err (the result of that scan is then wrong and the batch reports an error).
// state[0] holds the ticket counter, state[1 + t] tile t's word; the launcher zeroes them.
//
// Each warp owns 1024 consecutive elements of its tile and moves them as 8 rows of 32 x uint4
// (every load and store instruction of a warp covers 512 contiguous bytes). `Src::get4(i)` gives
// elements i..i+3 (zero past the end), `Dst::put4(i, excl, val)` receives their exclusive
// prefixes and values, so producers and consumers of a scan can be fused into it.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kLbThreads = 256;
constexpr uint32_t kLbRows = 8;
constexpr uint32_t kLbWarpSpan = kLbRows * 32u * 4u;           // 1024 elements per warp
constexpr uint32_t kLbTile = (kLbThreads / 32u) * kLbWarpSpan; // 8192 elements per tile
constexpr unsigned long long kLbAgg = 1ull << 62, kLbPre = 2ull << 62;

__device__ __forceinline__ unsigned long long ld_status(const unsigned long long* p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_status(unsigned long long* p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive prefix of the tile `tile` whose own total is `total` (warp 0 of the block; the
// result is valid in every lane).
__device__ __forceinline__ uint32_t lb_tile_prefix(unsigned long long* tiles, uint32_t tile, uint32_t total,
                                                   uint32_t* err, uint32_t poll_limit)
{
    const uint32_t lane = lane_id();
    if (tile == 0)
    {
        if (lane == 0)
            st_status(&tiles[0], kLbPre | total);
        return 0u;
    }
    if (lane == 0)
        st_status(&tiles[tile], kLbAgg | total);
    uint32_t prefix = 0;
    bool ok = true;
    for (int64_t hi = static_cast<int64_t>(tile) - 1; hi >= 0; hi -= 32)
    {
        const int64_t t = hi - static_cast<int64_t>(lane);
        unsigned long long w = kLbPre; // lanes past tile 0 contribute nothing
        if (t >= 0)
        {
            uint32_t polls = 0;
            do
                w = ld_status(&tiles[t]);
            while ((w >> 62) == 0u && ++polls < poll_limit);
            if ((w >> 62) == 0u)
            {
                ok = false;
                w = kLbPre;
            }
        }
        const uint32_t pre = __ballot_sync(0xffffffffu, (w >> 62) == 2u);
        const uint32_t upto = pre ? static_cast<uint32_t>(__ffs(pre) - 1) : 31u; // nearest prefix
        const uint32_t val = (lane <= upto) ? static_cast<uint32_t>(w) : 0u;
        prefix += warp_sum(val);
        if (pre)
            break;
    }
    if (!__all_sync(0xffffffffu, ok) && lane == 0 && err)
        atomicOr(err, static_cast<uint32_t>(ERR_INTERNAL));
    if (lane == 0)
        st_status(&tiles[tile], kLbPre | (prefix + total));
    return prefix;
}

constexpr uint32_t kLbPollLimit = 1u << 24; // polls of a predecessor's word before giving up

template <class Src, class Dst>
__global__ void __launch_bounds__(kLbThreads) k_scan_lb(Src src, Dst dst, unsigned long long* state, uint32_t* err,
                                                        uint32_t poll_limit)
{
    __shared__ uint32_t s_warp[kLbThreads / 32];
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0)
        s_tile = atomicAdd(reinterpret_cast<unsigned int*>(state), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const uint32_t wbase = tile * kLbTile + warp * kLbWarpSpan;
    uint4 v[kLbRows];
#pragma unroll
    for (uint32_t q = 0; q < kLbRows; ++q)
        v[q] = src.get4(wbase + (q * 32u + lane) * 4u);
    uint32_t rowx[kLbRows]; // exclusive prefix of this lane's 4 elements within the warp's span
    uint32_t wrun = 0;
#pragma unroll
    for (uint32_t q = 0; q < kLbRows; ++q)
    {
        const uint32_t sq = v[q].x + v[q].y + v[q].z + v[q].w;
        const uint32_t inc = warp_incl_scan(sq);
        rowx[q] = wrun + inc - sq;
        wrun += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0)
        s_warp[warp] = wrun;
    __syncthreads();
    if (warp == 0)
    {
        const uint32_t wv = (lane < kLbThreads / 32) ? s_warp[lane] : 0u;
        const uint32_t wi = warp_incl_scan(wv);
        const uint32_t total = __shfl_sync(0xffffffffu, wi, 31);
        const uint32_t prefix = lb_tile_prefix(state + 1, tile, total, err, poll_limit);
        if (lane < kLbThreads / 32)
            s_warp[lane] = prefix + wi - wv;
    }
    __syncthreads();
    const uint32_t wpre = s_warp[warp];
#pragma unroll
    for (uint32_t q = 0; q < kLbRows; ++q)
    {
        uint4 e;
        e.x = wpre + rowx[q];
        e.y = e.x + v[q].x;
        e.z = e.y + v[q].y;
        e.w = e.z + v[q].z;
        dst.put4(wbase + (q * 32u + lane) * 4u, e, v[q]);
    }
}

template <class Src, class Dst>
void scan_lookback(cudaStream_t st, Src src, Dst dst, uint32_t n, uint32_t* sums, uint32_t* err)
{
    const uint32_t nt = div_up(n, kLbTile);
    unsigned long long* state = reinterpret_cast<unsigned long long*>(sums);
    cudaMemsetAsync(state, 0, (static_cast<size_t>(nt) + 1) * sizeof(unsigned long long), st);
    k_scan_lb<<<nt, kLbThreads, 0, st>>>(src, dst, state, err, kLbPollLimit);
}

// Plain u32 arrays as scan source and destination (vector accesses when 16-byte aligned).
struct ScanSrcU32
{
    const uint32_t* p;
    uint32_t n;
    bool vec;
    __device__ __forceinline__ uint4 get4(uint32_t i) const
    {
        if (vec && i + 4u <= n)
            return *reinterpret_cast<const uint4*>(p + i);
        uint4 r;
        r.x = (i < n) ? p[i] : 0u;
        r.y = (i + 1u < n) ? p[i + 1u] : 0u;
        r.z = (i + 2u < n) ? p[i + 2u] : 0u;
        r.w = (i + 3u < n) ? p[i + 3u] : 0u;
        return r;
    }
};
struct ScanDstU32
{
    uint32_t* p;
    uint32_t n;
    bool vec;
    __device__ __forceinline__ void put4(uint32_t i, uint4 e, uint4) const
    {
        if (vec && i + 4u <= n)
        {
            *reinterpret_cast<uint4*>(p + i) = e;
            return;
        }
        if (i < n)
            p[i] = e.x;
        if (i + 1u < n)
            p[i + 1u] = e.y;
        if (i + 2u < n)
            p[i + 2u] = e.z;
        if (i + 3u < n)
            p[i + 3u] = e.w;
    }
};
} // namespace lpg
