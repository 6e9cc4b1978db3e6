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
} // namespace lpg
