// lp_introsort.cuh — libstdc++'s std::sort (introsort) replayed on the device by one CTA, for the
// reference's hull tie order (Polygonizer::convexHull sorts point indices with std::sort,
// polygonizer.cpp:51-59; which of several identical points ends up on the hull depends on the
// order std::sort leaves them in).
//
// The sequence GCC's <bits/stl_algo.h> performs: introsort_loop on ranges above 16 elements (depth
// limit 2 floor(log2 n); pivot = median of a[first + 1], a[mid], a[last - 1] swapped into a[first];
// unguarded Hoare partition of [first + 1, last); both sides continue with the decremented depth;
// heapsort of a range whose depth reaches 0), then the final insertion sort. The final pass equals
// an insertion sort of each leaf range on its own: no element crosses a partition cut (every
// element left of a cut is not greater than the pivot, every element right of it not less), and
// insertion sort never moves an element past an equal one. So disjoint ranges can be processed in
// any order and in parallel.
//
// One partition is replayed in parallel: with ge (le) the ascending positions of the elements
// >= (<=) the pivot in [first + 1, last), the t-th left stop ge[t - 1] is swapped with the t-th right
// stop le[nle - t] while ge[t - 1] < le[nle - t] (T swaps), and the scan stops at
// min(ge[T], le[nle - T]). Ranges above kCtaMin are partitioned by the whole CTA, one at a time;
// smaller ones are collected into batches that the warps process level by level (one range per
// warp, ballots for the lists, a 32-way search for T). A leaf range (at most 16 elements) is marked
// in the ge list area at its first position, which no later partition touches, and all leaves are
// insertion-sorted in parallel at the end.
#pragma once
#include <cstdint>

namespace lpg
{
namespace isort
{
constexpr uint32_t kSortLeaf = 16;                            // libstdc++'s _S_threshold
constexpr uint32_t kCtaMin = 2048;                            // ranges above: partitioned by the whole CTA
constexpr uint32_t kLevelCap = 512;                           // ranges of one level of a batch
constexpr uint32_t kBatchMax = kLevelCap * (kSortLeaf + 1);   // a batch's total length: <= kLevelCap ranges above 16
constexpr uint32_t kBatchFlush = kBatchMax - 2 * kCtaMin;     // room for the two children of one more CTA partition
constexpr uint32_t kBigCap = 64;                              // depth-first stack of CTA ranges (<= 2 log2 n pending)
constexpr uint32_t kLeafFlag = 0x80000000u;

// The sort's shared state; the caller declares one per CTA (about 17 KB).
struct SortShared
{
    uint4 lvl[2][kLevelCap]; // a batch's ranges of the current and the next level: first, last, depth
    uint4 big[kBigCap];
    uint32_t nlvl[2], nbig, batch_len;
    uint32_t words[40];      // partition_block: warp sums and the broadcast (blockDim / 32 + 4 <= 40)
};

__device__ __forceinline__ int floor_log2(uint32_t v)
{
    return 31 - __clz(v);
}

template <class T>
__device__ __forceinline__ void swap_at(T* a, uint32_t i, uint32_t j)
{
    const T t = a[i];
    a[i] = a[j];
    a[j] = t;
}

template <class T, class Less>
__device__ void median_to_first(T* a, uint32_t first, uint32_t last, Less less)
{
    const uint32_t x = first + 1, y = first + (last - first) / 2, z = last - 1;
    uint32_t m;
    if (less(a[x], a[y]))
        m = less(a[y], a[z]) ? y : (less(a[x], a[z]) ? z : x);
    else
        m = less(a[x], a[z]) ? x : (less(a[y], a[z]) ? z : y);
    swap_at(a, first, m);
}

// std::__adjust_heap + __push_heap on a[base, base + len).
template <class T, class Less>
__device__ void sift(T* a, uint32_t base, uint32_t hole, uint32_t len, T v, Less less)
{
    const uint32_t top = hole;
    uint32_t child = hole;
    while (len >= 2 && child < (len - 1) / 2)
    {
        child = 2 * (child + 1);
        if (less(a[base + child], a[base + child - 1]))
            --child;
        a[base + hole] = a[base + child];
        hole = child;
    }
    if ((len & 1u) == 0 && len >= 2 && child == (len - 2) / 2)
    {
        child = 2 * (child + 1);
        a[base + hole] = a[base + child - 1];
        hole = child - 1;
    }
    uint32_t parent = (hole - 1) / 2;
    while (hole > top && less(a[base + parent], v))
    {
        a[base + hole] = a[base + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[base + hole] = v;
}

// std::__partial_sort(first, last, last): make_heap, then pop into place (the depth-limit path).
template <class T, class Less>
__device__ void heap_sort(T* a, uint32_t first, uint32_t last, Less less)
{
    const uint32_t len = last - first;
    if (len < 2)
        return;
    for (uint32_t parent = (len - 2) / 2;; --parent)
    {
        sift(a, first, parent, len, a[first + parent], less);
        if (parent == 0)
            break;
    }
    for (uint32_t l = len - 1; l > 0; --l)
    {
        const T v = a[first + l];
        a[first + l] = a[first];
        sift(a, first, 0, l, v, less);
    }
}

// Insertion sort of [first, last) (std::__insertion_sort).
template <class T, class Less>
__device__ void insertion(T* a, uint32_t first, uint32_t last, Less less)
{
    if (first == last)
        return;
    for (uint32_t i = first + 1; i < last; ++i)
    {
        const T v = a[i];
        if (less(v, a[first]))
        {
            for (uint32_t j = i; j > first; --j)
                a[j] = a[j - 1];
            a[first] = v;
        }
        else
        {
            uint32_t j = i;
            while (j > first + 1 && less(v, a[j - 1]))
            {
                a[j] = a[j - 1];
                --j;
            }
            a[j] = v;
        }
    }
}

// One partition of [first, last) by one warp (all 32 lanes). ge/le: list areas indexed by position
// (the range's own entries [first, last) are used). Returns the cut.
template <class T, class Less>
__device__ uint32_t partition_warp(T* a, uint32_t first, uint32_t last, Less less, uint32_t* ge, uint32_t* le)
{
    const uint32_t lane = threadIdx.x & 31u, below = (1u << lane) - 1u;
    if (lane == 0)
        median_to_first(a, first, last, less);
    __syncwarp();
    const T p = a[first];
    const uint32_t lo = first + 1, n = last - lo;
    uint32_t nge = 0, nle = 0;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t idx = base + lane;
        bool g = false, l = false;
        if (idx < n)
        {
            const T v = a[lo + idx];
            g = !less(v, p);
            l = !less(p, v);
        }
        const uint32_t bg = __ballot_sync(0xffffffffu, g), bl = __ballot_sync(0xffffffffu, l);
        if (g)
            ge[first + nge + static_cast<uint32_t>(__popc(bg & below))] = lo + idx;
        if (l)
            le[first + nle + static_cast<uint32_t>(__popc(bl & below))] = lo + idx;
        nge += static_cast<uint32_t>(__popc(bg));
        nle += static_cast<uint32_t>(__popc(bl));
    }
    __syncwarp();
    // T: the largest t with ge[t - 1] < le[nle - t] (true up to T, false after), 32 candidates a round
    uint32_t tlo = 0, thi = min(nge, nle);
    while (tlo < thi)
    {
        const uint32_t step = (thi - tlo + 31u) / 32u;
        const uint32_t t = tlo + (lane + 1u) * step;
        const bool ok = t <= thi && ge[first + t - 1u] < le[first + nle - t];
        const uint32_t k = static_cast<uint32_t>(__popc(__ballot_sync(0xffffffffu, ok)));
        thi = min(thi, tlo + (k + 1u) * step - 1u);
        tlo += k * step;
    }
    const uint32_t swaps = tlo;
    const uint32_t cut = (swaps == 0) ? ge[first]
                                      : min(swaps < nge ? ge[first + swaps] : 0xffffffffu, le[first + nle - swaps]);
    for (uint32_t t = lane; t < swaps; t += 32)
        swap_at(a, ge[first + t], le[first + nle - 1u - t]);
    __syncwarp();
    return cut;
}

// One partition of [first, last) by the whole CTA (median of three by thread 0). ge/le as for
// partition_warp; words: blockDim / 32 + 4 shared words. Returns the cut.
template <class T, class Less>
__device__ uint32_t partition_block(T* a, uint32_t first, uint32_t last, Less less, uint32_t* ge, uint32_t* le,
                                    uint32_t* words)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
    uint32_t* warp_sum = words;
    uint32_t* bcast = words + nwarps;
    if (tid == 0)
        median_to_first(a, first, last, less);
    __syncthreads();
    const T p = a[first];
    const uint32_t lo = first + 1, n = last - lo, below = (1u << lane) - 1u;
    uint32_t nge = 0, nle = 0;
    for (uint32_t base = 0; base < n; base += blockDim.x)
    {
        const uint32_t idx = base + tid;
        bool g = false, l = false;
        if (idx < n)
        {
            const T v = a[lo + idx];
            g = !less(v, p);
            l = !less(p, v);
        }
        const uint32_t bg = __ballot_sync(0xffffffffu, g), bl = __ballot_sync(0xffffffffu, l);
        if (lane == 0)
            warp_sum[warp] = static_cast<uint32_t>(__popc(bg)) | (static_cast<uint32_t>(__popc(bl)) << 16);
        __syncthreads();
        uint32_t pre_g = 0, pre_l = 0, tot_g = 0, tot_l = 0;
        for (uint32_t w = 0; w < nwarps; ++w)
        {
            const uint32_t v = warp_sum[w];
            if (w < warp)
            {
                pre_g += v & 0xffffu;
                pre_l += v >> 16;
            }
            tot_g += v & 0xffffu;
            tot_l += v >> 16;
        }
        if (g)
            ge[first + nge + pre_g + static_cast<uint32_t>(__popc(bg & below))] = lo + idx;
        if (l)
            le[first + nle + pre_l + static_cast<uint32_t>(__popc(bl & below))] = lo + idx;
        nge += tot_g;
        nle += tot_l;
        __syncthreads();
    }
    if (tid == 0)
    {
        uint32_t lo_t = 0, hi_t = min(nge, nle);
        while (lo_t < hi_t)
        {
            const uint32_t mid = (lo_t + hi_t + 1) / 2;
            if (ge[first + mid - 1] < le[first + nle - mid])
                lo_t = mid;
            else
                hi_t = mid - 1;
        }
        bcast[0] = lo_t;
        bcast[1] = (lo_t == 0) ? ge[first]
                               : min(lo_t < nge ? ge[first + lo_t] : 0xffffffffu, le[first + nle - lo_t]);
    }
    __syncthreads();
    const uint32_t swaps = bcast[0], cut = bcast[1];
    for (uint32_t t = tid; t < swaps; t += blockDim.x)
        swap_at(a, ge[first + t], le[first + nle - 1 - t]);
    __syncthreads();
    return cut;
}

// A child range of a partition: a leaf is marked for the final insertion pass; a range that
// still needs partitioning is returned true (the caller queues it).
__device__ __forceinline__ bool leaf_or_queue(uint32_t f, uint32_t l, uint32_t* ge)
{
    if (l - f > kSortLeaf)
        return true;
    if (l - f > 1)
        ge[f] = kLeafFlag | l;
    return false;
}

// The batch in ss.lvl[0] (ss.nlvl[0] ranges, each above 16 and at most kCtaMin, total length at
// most kBatchMax), level by level: warp w partitions ranges w, w + nwarps, ... of the level and
// queues their children on the next one.
template <class T, class Less>
__device__ void run_batch(T* a, Less less, uint32_t* ge, uint32_t* le, SortShared& ss)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int cur = 0;
    __syncthreads();
    while (ss.nlvl[cur] > 0)
    {
        const uint32_t cnt = ss.nlvl[cur];
        if (threadIdx.x == 0)
            ss.nlvl[cur ^ 1] = 0;
        __syncthreads();
        for (uint32_t k = warp; k < cnt; k += nwarps)
        {
            const uint4 r = ss.lvl[cur][k];
            if (r.z == 0)
            {
                if (lane == 0)
                    heap_sort(a, r.x, r.y, less); // the depth limit (not reached on real clouds)
                __syncwarp();
                continue;
            }
            const uint32_t cut = partition_warp(a, r.x, r.y, less, ge, le);
            if (lane < 2)
            {
                const uint32_t f = lane ? cut : r.x, l = lane ? r.y : cut;
                if (leaf_or_queue(f, l, ge))
                    ss.lvl[cur ^ 1][atomicAdd(&ss.nlvl[cur ^ 1], 1u)] = make_uint4(f, l, r.z - 1u, 0u);
            }
            __syncwarp();
        }
        __syncthreads();
        cur ^= 1;
    }
    if (threadIdx.x == 0)
    {
        ss.nlvl[0] = 0;
        ss.batch_len = 0;
    }
    __syncthreads();
}

// std::sort(a, a + n, less) by one CTA (blockDim a multiple of 32, at most 1024). ge/le: n words
// each (global or shared memory). The result is the element order libstdc++'s std::sort leaves.
template <class T, class Less>
__device__ void cta_sort(T* a, uint32_t n, Less less, uint32_t* ge, uint32_t* le, SortShared& ss)
{
    if (n < 2)
        return;
    for (uint32_t p = threadIdx.x; p < n; p += blockDim.x)
        ge[p] = 0; // no leaf marks yet
    const uint32_t depth0 = static_cast<uint32_t>(2 * floor_log2(n));
    if (threadIdx.x == 0)
    {
        ss.nbig = 0;
        ss.nlvl[0] = 0;
        ss.batch_len = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (n > kCtaMin)
            ss.big[ss.nbig++] = make_uint4(0u, n, depth0, 0u);
        else if (leaf_or_queue(0u, n, ge))
        {
            ss.lvl[0][ss.nlvl[0]++] = make_uint4(0u, n, depth0, 0u);
            ss.batch_len = n;
        }
    }
    __syncthreads();
    while (ss.nbig > 0)
    {
        const uint4 r = ss.big[ss.nbig - 1];
        __syncthreads();
        if (threadIdx.x == 0)
            --ss.nbig;
        __syncthreads();
        if (r.z == 0)
        {
            if (threadIdx.x == 0)
                heap_sort(a, r.x, r.y, less); // the depth limit (not reached on real clouds)
            __syncthreads();
            continue;
        }
        const uint32_t cut = partition_block(a, r.x, r.y, less, ge, le, ss.words);
        if (threadIdx.x == 0)
        {
            const uint4 kids[2] = {make_uint4(r.x, cut, r.z - 1u, 0u), make_uint4(cut, r.y, r.z - 1u, 0u)};
            for (const uint4& k : kids)
            {
                if (k.y - k.x > kCtaMin && ss.nbig < kBigCap)
                    ss.big[ss.nbig++] = k;
                else if (k.y - k.x > kCtaMin)
                    heap_sort(a, k.x, k.y, less); // stack full: unreachable, depth <= 2 log2 n < kBigCap
                else if (leaf_or_queue(k.x, k.y, ge))
                {
                    ss.lvl[0][ss.nlvl[0]++] = k;
                    ss.batch_len += k.y - k.x;
                }
            }
        }
        __syncthreads();
        if (ss.batch_len > kBatchFlush)
            run_batch(a, less, ge, le, ss);
    }
    run_batch(a, less, ge, le, ss);
    for (uint32_t p = threadIdx.x; p < n; p += blockDim.x)
    {
        const uint32_t v = ge[p];
        if (v & kLeafFlag)
            insertion(a, p, v & ~kLeafFlag, less);
    }
    __syncthreads();
}
} // namespace isort
} // namespace lpg
