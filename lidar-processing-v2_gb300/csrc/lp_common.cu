// lp_common.cu — device-wide exclusive scan (single pass, decoupled look-back).
#include "lp_common.cuh"

namespace lpg
{
// ---------------------------------------------------------------------------------------------
// Single-pass exclusive scan with decoupled look-back (Merrill & Garland, "Single-pass Parallel
// Prefix Scan with Decoupled Look-back", 2016). Tiles of kLbTile elements take dynamic tickets, so
// every tile a block waits for has already started (and waits only for earlier ones): each
// look-back ends. A tile publishes (flag, value) in one 64-bit word: flag 1 = the tile's own sum,
// flag 2 = the inclusive prefix through the tile. Waits are bounded anyway; running out sets
// ERR_INTERNAL in *err (the result of that scan is then wrong and the batch reports an error).
// state[0] holds the ticket counter, state[1 + t] tile t's word; the caller zeroes
// 1 + ntiles words before each scan.
// ---------------------------------------------------------------------------------------------
constexpr uint32_t kLbThreads = 256;
constexpr uint32_t kLbItems = 32;
constexpr uint32_t kLbTile = kLbThreads * kLbItems;
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

__global__ void __launch_bounds__(kLbThreads) k_scan_lookback(const uint32_t* in, uint32_t* out, uint32_t n,
                                                              unsigned long long* state, uint32_t* err)
{
    __shared__ uint32_t sm[33];
    __shared__ uint32_t s_tile, s_prefix;
    if (threadIdx.x == 0)
        s_tile = atomicAdd(reinterpret_cast<unsigned int*>(state), 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * kLbTile + threadIdx.x * kLbItems;
    uint32_t v[kLbItems];
    const bool vec = base + kLbItems <= n &&
                     ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0u;
    if (vec)
    {
        const uint4* p = reinterpret_cast<const uint4*>(in + base);
#pragma unroll
        for (uint32_t q = 0; q < kLbItems / 4; ++q)
        {
            const uint4 w = p[q];
            v[4 * q] = w.x;
            v[4 * q + 1] = w.y;
            v[4 * q + 2] = w.z;
            v[4 * q + 3] = w.w;
        }
    }
    else
    {
#pragma unroll
        for (uint32_t k = 0; k < kLbItems; ++k)
            v[k] = (base + k < n) ? in[base + k] : 0u;
    }
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < kLbItems; ++k)
        sum += v[k];
    uint32_t total;
    const uint32_t excl = block_excl_scan(sum, sm, &total);
    unsigned long long* tiles = state + 1;
    if (threadIdx.x < 32)
    {
        const uint32_t lane = threadIdx.x;
        uint32_t prefix = 0;
        if (tile == 0)
        {
            if (lane == 0)
                st_status(&tiles[0], kLbPre | total);
        }
        else
        {
            if (lane == 0)
                st_status(&tiles[tile], kLbAgg | total);
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
                    while ((w >> 62) == 0u && ++polls < (1u << 24));
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
        }
        if (lane == 0)
            s_prefix = prefix;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
    if (vec)
    {
        uint4* p = reinterpret_cast<uint4*>(out + base);
#pragma unroll
        for (uint32_t q = 0; q < kLbItems / 4; ++q)
        {
            uint4 w;
            w.x = run;
            run += v[4 * q];
            w.y = run;
            run += v[4 * q + 1];
            w.z = run;
            run += v[4 * q + 2];
            w.w = run;
            run += v[4 * q + 3];
            p[q] = w;
        }
    }
    else
    {
#pragma unroll
        for (uint32_t k = 0; k < kLbItems; ++k)
        {
            if (base + k < n)
                out[base + k] = run;
            run += v[k];
        }
    }
}

// Exclusive scan of n u32 (in place allowed). `sums` is the scan scratch (at least
// 8 * (div_up(n, 4096) + 2) bytes, 8-byte aligned), `err` the error word (or null).
void scan_exclusive(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* err,
                    uint64_t& launches)
{
    const uint32_t nt = div_up(n, kLbTile);
    unsigned long long* state = reinterpret_cast<unsigned long long*>(sums);
    cudaMemsetAsync(state, 0, (static_cast<size_t>(nt) + 1) * sizeof(unsigned long long), st);
    k_scan_lookback<<<nt, kLbThreads, 0, st>>>(in, out, n, state, err);
    launches += 1;
}
} // namespace lpg
