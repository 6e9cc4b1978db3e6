// lp_common.cu — device-wide exclusive scan (reduce / scan partials / downsweep).
#include "lp_common.cuh"

namespace lpg
{
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* __restrict__ in, uint32_t n,
                                                             uint32_t* __restrict__ sums)
{
    __shared__ uint32_t sm[33];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n)
            s += in[base + k];
    s = warp_sum(s);
    if (lane_id() == 0)
        sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        uint32_t t = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w)
            t += sm[w];
        sums[blockIdx.x] = t;
    }
}

// One block: exclusive scan of the per-tile sums in place, total to *grand_total.
__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* sums, uint32_t nb, uint32_t* grand_total)
{
    __shared__ uint32_t sm[33];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += blockDim.x)
    {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = (i < nb) ? sums[i] : 0u;
        const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
        const uint32_t incl = warp_incl_scan(v);
        if (lane == 31)
            sm[warp] = incl;
        __syncthreads();
        if (warp == 0)
        {
            const uint32_t w = sm[lane];
            const uint32_t wi = warp_incl_scan(w);
            sm[lane] = wi - w;
            if (lane == 31)
                sm[32] = wi;
        }
        __syncthreads();
        if (i < nb)
            sums[i] = carry + sm[warp] + incl - v;
        carry += sm[32];
        __syncthreads();
    }
    if (threadIdx.x == 0 && grand_total)
        *grand_total = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t* in, uint32_t* out, uint32_t n,
                                                           const uint32_t* __restrict__ sums)
{
    __shared__ uint32_t sm[33];
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
    {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t total;
    uint32_t pre = block_excl_scan(s, sm, &total) + sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
    {
        if (base + k < n)
            out[base + k] = pre;
        pre += v[k];
    }
}

void scan_exclusive(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums,
                    uint32_t* grand_total, uint64_t& launches)
{
    const uint32_t nb = div_up(n, static_cast<uint32_t>(kScanTile));
    k_scan_reduce<<<nb, kScanThreads, 0, st>>>(in, n, sums);
    k_scan_sums<<<1, 1024, 0, st>>>(sums, nb, grand_total);
    k_scan_down<<<nb, kScanThreads, 0, st>>>(in, out, n, sums);
    launches += 3;
}
} // namespace lpg
