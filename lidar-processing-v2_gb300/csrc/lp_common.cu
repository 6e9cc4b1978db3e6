// lp_common.cu — device-wide exclusive scan of u32 arrays (the look-back kernel is in lp_common.cuh).
#include "lp_common.cuh"

namespace lpg
{
// Exclusive scan of n u32 (in place allowed). `sums` is the scan scratch (at least
// 8 * (div_up(n, 4096) + 2) bytes, 8-byte aligned), `err` the error word (or null).
void scan_exclusive(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* err,
                    uint64_t& launches)
{
    const bool vec = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) == 0u;
    scan_lookback(st, ScanSrcU32{in, n, vec}, ScanDstU32{out, n, vec}, n, sums, err);
    launches += 1;
}

namespace
{
// A wait that nothing will satisfy, to check that bounded waits give up and report: an mbarrier
// expecting one arrival that never comes, polled `limit` times.
__global__ void k_debug_mbar_timeout(uint32_t limit, uint32_t* err)
{
    __shared__ unsigned long long bar;
    if (threadIdx.x == 0)
        mbar_init(&bar, 1u);
    __syncthreads();
    if (!mbar_wait(&bar, 0u, limit) && threadIdx.x == 0)
        atomicOr(err, static_cast<uint32_t>(ERR_INTERNAL));
}
} // namespace

// kind 0: a look-back scan over one tile whose ticket counter starts at 1, so its only block takes
// tile 1 and waits for tile 0's word, which no block writes (every element lies past n: nothing is
// read or written besides the state words); kind 1: an mbarrier wait without an arrival. Both give
// up after `limit` polls and set ERR_INTERNAL in *err. `state` holds at least 4 words.
void launch_debug_wait_timeout(cudaStream_t st, int kind, uint32_t limit, unsigned long long* state, uint32_t* err,
                               uint64_t& launches)
{
    if (kind == 0)
    {
        const unsigned long long start[4] = {1ull, 0ull, 0ull, 0ull};
        cudaMemcpyAsync(state, start, sizeof(start), cudaMemcpyHostToDevice, st);
        k_scan_lb<<<1, kLbThreads, 0, st>>>(ScanSrcU32{nullptr, 0u, false}, ScanDstU32{nullptr, 0u, false}, state, err,
                                            limit);
    }
    else
    {
        k_debug_mbar_timeout<<<1, 32, 0, st>>>(limit, err);
    }
    launches += 1;
}
} // namespace lpg
