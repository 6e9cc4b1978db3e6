// lp_kdtree.cu — dynamic-radius outlier removal exactly as the reference's kd-tree search leaves it.
//
// Reference: NoiseRemover::filter (lidar_processing_lib/src/noise_remover.cpp:38-68) over
// KDTree::rebuild (kdtree.hpp:161-214) and KDTree::radius_search_k_nearest (kdtree.hpp:339-397).
// Per point, in input order: squared radius r2 = max(float(s2 * double(x*x + y*y)), rmin^2); a
// depth-first search from the root counts nodes with d0 + (d1 + d2) <= r2 (dk = (q_k - p_k)^2 in
// binary32, query first) and stops at min_neighbours; fewer found means NOISE. The search's stack
// is a member of the tree and is not cleared when the search stops early: the next point's search
// pushes the root on top of what is left, and once its own subtrees are exhausted it carries on
// through the subtrees earlier searches left behind, counting points there again. A point with
// fewer than min_neighbours true neighbours can therefore still reach the count. This file
// reproduces that sequence exactly (every scan starts with an empty stack, as a new NoiseRemover):
//
//   1. Tree (k_kt_level): the reference builds its tree by std::nth_element on the middle of
//      each range (x, y, z by depth); which of several points with equal coordinates lands on
//      which side depends on that library routine's swaps. The build replays libstdc++'s
//      introselect step for step (median of three, unguarded Hoare partition, insertion sort at
//      three elements, heap selection at the depth limit). Large ranges: one CTA per range, the
//      Hoare partition replayed in parallel (the t-th element >= pivot from the left is swapped
//      with the t-th element <= pivot from the right while the first lies left of the second);
//      ranges of at most kKtSmall points finish their whole subtree in shared memory. Node
//      children follow from the range arithmetic alone, so a node record is its point and its
//      subtree size; subtree boxes (k_kt_box_level) serve the skip test of steps 3 and 4.
//   2. Own search (k_kt_own, one thread per point, taken in tree order): the point's search from
//      the root, in the reference's push order, until min_neighbours or exhaustion. A point that reaches the
//      count leaves the rest of its stack behind: those entries go to a pool, then into one
//      array in point order (k_kt_flat). Points that exhaust their own search ("short" points)
//      are listed in order (k_kt_short).
//   3. Own segment (k_kt_segment, one thread per short point): the stack a short point meets is
//      the leftovers of the points since the previous short point (a contiguous piece of the
//      array, newest on top) above whatever the previous short point left. The point walks its
//      piece from the top; an entry whose subtree box is farther than the radius is consumed
//      without a match (skipped); the others are searched exactly. Reaching the count there
//      decides the point (VALID) and records where it stopped and the entries it left.
//   4. Candidates (short points step 3 did not decide) in three steps. k_kt_spec, one thread per
//      candidate: the walk through the pieces pushed since the previous candidate, as if nothing
//      lay below them, which is exact whenever the previous candidate emptied the stack (running
//      out of entries is NOISE). k_kt_spec_next, one thread per candidate whose walk ran out right
//      after one whose walk stopped: the walk on through the pieces that stop leaves, which lie
//      on top of whatever was below. k_kt_chain, one CTA per scan: the candidates in order with R,
//      what earlier walks left below those pieces; a stopped walk adds its remainder to R, one
//      that ran out continues into R: straight after a stop with the walk k_kt_spec_next made,
//      otherwise (and below those pieces) with the threads searching 256 entries at a time, an
//      ordered prefix of their counts finding the stop. While R is empty, runs of candidates whose
//      walks ran out are NOISE at once.
// The result equals the reference's sequential search bit for bit (same binary32 expressions,
// same visiting order, same stop points); the tree's node positions equal the reference's.
#include <cooperative_groups.h>

#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace cg = cooperative_groups;

namespace lpg
{
namespace
{
constexpr uint32_t kKtSmall = 2048;    // ranges built in shared memory by one CTA
constexpr uint32_t kKtHuge = 65536;    // ranges partitioned by a cluster of kKtCluster CTAs
constexpr uint32_t kKtClusterMin = 8192; // the cluster's rounds run while the range exceeds this
constexpr int kKtCluster = 8;
constexpr uint32_t kKtWarpMin = 16;    // ranges of at most this many points finish on one thread
constexpr int kKtThreads = 512;        // tree build CTAs
constexpr int kKtItems = 8;            // elements per thread per tile of the parallel partition
constexpr int kKtStack = 64;           // search stack entries (>= tree depth + 1 for 2^62 points)
constexpr uint32_t kNone = 0xffffffffu;

// Stack entries: node position (scan-local) << 2 | axis.
__device__ __forceinline__ uint32_t kt_entry(uint32_t m, int ax)
{
    return (m << 2) | static_cast<uint32_t>(ax);
}

__device__ __forceinline__ float kt_coord(const float4& r, int ax)
{
    return ax == 0 ? r.x : (ax == 1 ? r.y : r.z);
}

__device__ __forceinline__ float kt_radius2(const ScanDev& sd, const float4& p)
{
    // noise_remover.cpp:55-57: float products and sum, widened, scaled, narrowed, floored
    const double rho2 = static_cast<double>((p.x * p.x) + (p.y * p.y));
    return fmaxf(__double2float_rn(sd.dror_s2 * rho2), sd.dror_rmin2);
}

__device__ __forceinline__ uint32_t floor_log2_u(uint32_t v)
{
    return 31u - static_cast<uint32_t>(__clz(v));
}

// Range of node slot j (0 <= j < 2^level) of the implicit tree over [0, n): the bits of j from the
// top choose left (0) or right (1) at each level. Returns false where the range does not exist.
// *plen receives the parent's length (n for the root).
__device__ __forceinline__ bool kt_range(uint32_t n, int level, uint32_t j, uint32_t& b, uint32_t& e, uint32_t* plen)
{
    b = 0;
    e = n;
    uint32_t parent = n;
    for (int l = level - 1; l >= 0; --l)
    {
        if (e <= b)
            return false;
        const uint32_t mid = b + (e - b) / 2;
        parent = e - b;
        if ((j >> l) & 1u)
            b = mid + 1;
        else
            e = mid;
    }
    if (plen)
        *plen = parent;
    return e > b;
}

// ---------------------------------------------------------------------------------------------
// libstdc++ introselect, one thread (std::nth_element as GCC's <bits/stl_algo.h> performs it).
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void kt_swap(float4* a, uint32_t i, uint32_t j)
{
    const float4 t = a[i];
    a[i] = a[j];
    a[j] = t;
}

// The median of a[first + 1], a[mid], a[last - 1] is swapped into a[first].
__device__ void kt_median_to_first(float4* a, uint32_t first, uint32_t last, int ax)
{
    const uint32_t x = first + 1, y = first + (last - first) / 2, z = last - 1;
    const float vx = kt_coord(a[x], ax), vy = kt_coord(a[y], ax), vz = kt_coord(a[z], ax);
    uint32_t m;
    if (vx < vy)
        m = (vy < vz) ? y : ((vx < vz) ? z : x);
    else
        m = (vx < vz) ? x : ((vy < vz) ? z : y);
    kt_swap(a, first, m);
}

// Unguarded Hoare partition of [first + 1, last) around a[first]; returns the cut. The median of
// three guarantees an element >= pivot and one <= pivot inside the range, which stop the scans;
// the explicit bounds only keep a malformed input (NaN coordinates) inside the range.
__device__ uint32_t kt_partition_seq(float4* a, uint32_t first, uint32_t last, int ax)
{
    const float p = kt_coord(a[first], ax);
    uint32_t lo = first + 1, hi = last;
    for (;;)
    {
        while (lo + 1 < last && kt_coord(a[lo], ax) < p)
            ++lo;
        --hi;
        while (hi > first && p < kt_coord(a[hi], ax))
            --hi;
        if (!(lo < hi))
            return lo;
        kt_swap(a, lo, hi);
        ++lo;
    }
}

__device__ void kt_insertion(float4* a, uint32_t first, uint32_t last, int ax)
{
    if (first == last)
        return;
    for (uint32_t i = first + 1; i < last; ++i)
    {
        const float4 v = a[i];
        const float kv = kt_coord(v, ax);
        if (kv < kt_coord(a[first], ax))
        {
            for (uint32_t j = i; j > first; --j)
                a[j] = a[j - 1];
            a[first] = v;
        }
        else
        {
            uint32_t j = i;
            while (j > first + 1 && kv < kt_coord(a[j - 1], ax))
            {
                a[j] = a[j - 1];
                --j;
            }
            a[j] = v;
        }
    }
}

// Max-heap sift of value v from `hole` in a[base, base + len) (std::__adjust_heap + __push_heap).
__device__ void kt_sift(float4* a, uint32_t base, uint32_t hole, uint32_t len, float4 v, int ax)
{
    const uint32_t top = hole;
    uint32_t child = hole;
    while (len >= 2 && child < (len - 1) / 2)
    {
        child = 2 * (child + 1);
        if (kt_coord(a[base + child], ax) < kt_coord(a[base + child - 1], ax))
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
    const float kv = kt_coord(v, ax);
    uint32_t parent = (hole - 1) / 2;
    while (hole > top && kt_coord(a[base + parent], ax) < kv)
    {
        a[base + hole] = a[base + parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    a[base + hole] = v;
}

// std::__heap_select(first, middle, last) then the swap of first and nth (introselect at the depth
// limit): a max-heap of [first, nth], every later element smaller than its top replaces it.
__device__ void kt_heap_select(float4* a, uint32_t first, uint32_t nth, uint32_t last, int ax)
{
    const uint32_t mid = nth - first + 1;
    if (mid >= 2)
        for (uint32_t parent = (mid - 2) / 2;; --parent)
        {
            kt_sift(a, first, parent, mid, a[first + parent], ax);
            if (parent == 0)
                break;
        }
    for (uint32_t i = first + mid; i < last; ++i)
        if (kt_coord(a[i], ax) < kt_coord(a[first], ax))
        {
            const float4 v = a[i];
            a[i] = a[first];
            kt_sift(a, first, 0, mid, v, ax);
        }
    kt_swap(a, first, nth);
}

// Continues an introselect of nth in [first, last) with `depth` rounds left, on one thread.
__device__ void kt_select_seq(float4* a, uint32_t first, uint32_t nth, uint32_t last, int depth, int ax)
{
    while (last - first > 3)
    {
        if (depth == 0)
        {
            kt_heap_select(a, first, nth, last, ax);
            return;
        }
        --depth;
        kt_median_to_first(a, first, last, ax);
        const uint32_t cut = kt_partition_seq(a, first, last, ax);
        if (cut <= nth)
            first = cut;
        else
            last = cut;
    }
    kt_insertion(a, first, last, ax);
}

// ---------------------------------------------------------------------------------------------
// One partition round by a whole CTA: median of three into a[first], then the unguarded Hoare
// partition of [first + 1, last) replayed in parallel. With L_t the t-th position (from the
// left) holding a value >= pivot and R_t the t-th (from the right) holding a value <= pivot, the
// sequential loop swaps L_t with R_t for every t with L_t < R_t (T such pairs; these pairs are
// disjoint) and then stops at min(L_{T+1}, R_T) (L_1 when T = 0): the left scan meets either the
// next original candidate or the element it swapped to R_T. ge/le receive the candidate
// positions in ascending order (le reversed gives R). Returns the cut.
// ---------------------------------------------------------------------------------------------
struct KtShared
{
    float tile[kKtThreads * kKtItems];
    uint32_t warp_sum[kKtThreads / 32];
    uint32_t bcast[4];
};

__device__ uint32_t kt_round_block(float4* a, uint32_t first, uint32_t last, int ax, uint32_t* ge, uint32_t* le,
                                   KtShared& sh)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const uint32_t nwarps = blockDim.x >> 5;
    if (tid == 0)
        kt_median_to_first(a, first, last, ax);
    __syncthreads();
    const float p = kt_coord(a[first], ax);
    const uint32_t lo = first + 1, n = last - lo;
    const uint32_t tile = blockDim.x * kKtItems;
    uint32_t nge = 0, nle = 0;
    for (uint32_t base = 0; base < n; base += tile)
    {
        const uint32_t cnt = min(tile, n - base);
        for (uint32_t k = tid; k < cnt; k += blockDim.x)
            sh.tile[k] = kt_coord(a[lo + base + k], ax);
        __syncthreads();
        uint32_t fge = 0, fle = 0, cge = 0, cle = 0;
#pragma unroll
        for (int k = 0; k < kKtItems; ++k)
        {
            const uint32_t idx = tid * kKtItems + k;
            if (idx < cnt)
            {
                const float v = sh.tile[idx];
                if (!(v < p))
                {
                    fge |= 1u << k;
                    ++cge;
                }
                if (!(p < v))
                {
                    fle |= 1u << k;
                    ++cle;
                }
            }
        }
        // block exclusive scan of (cge | cle << 16)
        const uint32_t packed = cge | (cle << 16);
        uint32_t incl = packed;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o))
                incl += t;
        }
        if (lane == 31)
            sh.warp_sum[warp] = incl;
        __syncthreads();
        uint32_t wpre = 0, total = 0;
        for (uint32_t w = 0; w < nwarps; ++w)
        {
            const uint32_t s = sh.warp_sum[w];
            if (w < warp)
                wpre += s;
            total += s;
        }
        const uint32_t ex = incl - packed + wpre;
        uint32_t og = nge + (ex & 0xffffu), ol = nle + (ex >> 16);
#pragma unroll
        for (int k = 0; k < kKtItems; ++k)
        {
            const uint32_t pos = lo + base + tid * kKtItems + k;
            if (fge & (1u << k))
                ge[og++] = pos;
            if (fle & (1u << k))
                le[ol++] = pos;
        }
        nge += total & 0xffffu;
        nle += total >> 16;
        __syncthreads();
    }
    // T: the largest t with ge[t - 1] < le[nle - t] (monotone in t)
    if (tid == 0)
    {
        uint32_t lo_t = 0, hi_t = min(nge, nle);
        while (lo_t < hi_t)
        {
            const uint32_t mid = (lo_t + hi_t + 1) / 2;
            if (ge[mid - 1] < le[nle - mid])
                lo_t = mid;
            else
                hi_t = mid - 1;
        }
        const uint32_t T = lo_t;
        uint32_t cut;
        if (T == 0)
            cut = ge[0];
        else
            cut = min(T < nge ? ge[T] : 0xffffffffu, le[nle - T]);
        sh.bcast[0] = T;
        sh.bcast[1] = cut;
    }
    __syncthreads();
    const uint32_t T = sh.bcast[0], cut = sh.bcast[1];
    for (uint32_t t = tid; t < T; t += blockDim.x)
        kt_swap(a, ge[t], le[nle - 1 - t]);
    __syncthreads();
    return cut;
}

__device__ void kt_select_warp(float4* a, uint32_t first, uint32_t nth, uint32_t last, int ax, uint16_t* ge,
                               uint16_t* le, int depth);

// Continues an introselect of nth in [first, last) (global memory) with `depth` rounds left on a
// whole CTA: parallel rounds while the range exceeds kKtSmall points, then the range is copied to
// shared memory (srec, with 2 kKtSmall list entries at slist) and warp 0 finishes it there. The
// depth-limit fallback on a larger range runs on thread 0.
__device__ void kt_select_block(float4* a, uint32_t first, uint32_t nth, uint32_t last, int depth, int ax,
                                uint32_t* ge, uint32_t* le, KtShared& sh, float4* srec, uint16_t* slist)
{
    while (last - first > kKtSmall && depth > 0)
    {
        --depth;
        const uint32_t cut = kt_round_block(a, first, last, ax, ge, le, sh);
        if (cut <= nth)
            first = cut;
        else
            last = cut;
    }
    const uint32_t len = last - first;
    if (len > kKtSmall)
    {
        if (threadIdx.x == 0)
            kt_select_seq(a, first, nth, last, depth, ax);
        __syncthreads();
        return;
    }
    for (uint32_t k = threadIdx.x; k < len; k += blockDim.x)
        srec[k] = a[first + k];
    __syncthreads();
    if (threadIdx.x < 32)
        kt_select_warp(srec, 0, nth - first, len, ax, slist, slist + len, depth);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < len; k += blockDim.x)
        a[first + k] = srec[k];
    __syncthreads();
}

// One partition round by one warp on a[first, last) in shared memory (the parallel Hoare replay of
// kt_round_block, 32 elements per step with ballots); ge/le hold the candidate positions.
__device__ uint32_t kt_round_warp(float4* a, uint32_t first, uint32_t last, int ax, uint16_t* ge, uint16_t* le)
{
    const uint32_t lane = lane_id();
    if (lane == 0)
        kt_median_to_first(a, first, last, ax);
    __syncwarp();
    const float p = kt_coord(a[first], ax);
    const uint32_t lo = first + 1, n = last - lo;
    const uint32_t below = (1u << lane) - 1u;
    uint32_t nge = 0, nle = 0;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t idx = base + lane;
        bool g = false, l = false;
        if (idx < n)
        {
            const float v = kt_coord(a[lo + idx], ax);
            g = !(v < p);
            l = !(p < v);
        }
        const uint32_t bg = __ballot_sync(0xffffffffu, g), bl = __ballot_sync(0xffffffffu, l);
        if (g)
            ge[nge + __popc(bg & below)] = static_cast<uint16_t>(lo + idx);
        if (l)
            le[nle + __popc(bl & below)] = static_cast<uint16_t>(lo + idx);
        nge += __popc(bg);
        nle += __popc(bl);
    }
    __syncwarp();
    uint32_t T = 0, cut = 0;
    if (lane == 0)
    {
        uint32_t lo_t = 0, hi_t = min(nge, nle);
        while (lo_t < hi_t)
        {
            const uint32_t mid = (lo_t + hi_t + 1) / 2;
            if (ge[mid - 1] < le[nle - mid])
                lo_t = mid;
            else
                hi_t = mid - 1;
        }
        T = lo_t;
        cut = (T == 0) ? ge[0] : min(T < nge ? static_cast<uint32_t>(ge[T]) : 0xffffffffu, static_cast<uint32_t>(le[nle - T]));
    }
    T = __shfl_sync(0xffffffffu, T, 0);
    cut = __shfl_sync(0xffffffffu, cut, 0);
    for (uint32_t t = lane; t < T; t += 32)
        kt_swap(a, ge[t], le[nle - 1 - t]);
    __syncwarp();
    return cut;
}

// Continues an introselect of nth in [first, last) (shared memory) with `depth` rounds left on one
// warp: parallel rounds while the range holds more than kKtWarpMin points, then lane 0 as written.
// (A parallel round replays the sequential partition exactly at any size; a small range on one
// thread is a chain of dependent shared-memory accesses, and ranges on neighbouring threads diverge.)
__device__ void kt_select_warp(float4* a, uint32_t first, uint32_t nth, uint32_t last, int ax, uint16_t* ge,
                               uint16_t* le, int depth)
{
    while (last - first > kKtWarpMin && depth > 0)
    {
        --depth;
        const uint32_t cut = kt_round_warp(a, first, last, ax, ge, le);
        if (cut <= nth)
            first = cut;
        else
            last = cut;
    }
    if (lane_id() == 0)
        kt_select_seq(a, first, nth, last, depth, ax);
    __syncwarp();
}

// Subtree of [b0, e0) (at depth d0 of the tree, at most kKtSmall points) built in shared memory;
// node records get their subtree size in .w (the input index it carried goes to idx); subtree
// boxes are written bottom-up.
__device__ void kt_build_small(float4* g, float4* box, uint32_t* idx, uint32_t b0, uint32_t e0, int d0, float4* s,
                               uint16_t* lists)
{
    const uint32_t n = e0 - b0;
    const uint32_t warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        s[k] = g[b0 + k];
    __syncthreads();
    // the longest range at depth d has floor(n / 2^d) points (a range of L splits into floor(L/2)
    // and ceil(L/2) - 1), so depths 0 .. floor(log2 n) hold ranges. Ranges above kKtWarpMin: one warp
    // each (positions of range [b, e) in lists[2b, 2e)); the rest: one thread each.
    const int maxd = static_cast<int>(floor_log2_u(n));
    for (int d = 0; d <= maxd; ++d)
    {
        const uint32_t slots = 1u << d;
        if ((n >> d) > kKtWarpMin)
            for (uint32_t j = warp; j < slots; j += nwarps)
            {
                uint32_t b, e;
                if (kt_range(n, d, j, b, e, nullptr) && e - b > kKtWarpMin)
                    kt_select_warp(s, b, b + (e - b) / 2, e, (d0 + d) % 3, lists + 2 * b, lists + 2 * b + (e - b),
                                   2 * static_cast<int>(floor_log2_u(e - b)));
            }
        for (uint32_t j = threadIdx.x; j < slots; j += blockDim.x)
        {
            uint32_t b, e;
            if (kt_range(n, d, j, b, e, nullptr) && e - b <= kKtWarpMin && e - b > 1)
                kt_select_seq(s, b, b + (e - b) / 2, e, 2 * static_cast<int>(floor_log2_u(e - b)), (d0 + d) % 3);
        }
        __syncthreads();
    }
    // subtree sizes and boxes, deepest level first
    for (int d = maxd; d >= 0; --d)
    {
        const uint32_t slots = 1u << d;
        for (uint32_t j = threadIdx.x; j < slots; j += blockDim.x)
        {
            uint32_t b, e;
            if (!kt_range(n, d, j, b, e, nullptr))
                continue;
            const uint32_t m = b + (e - b) / 2;
            float4 p = s[m];
            idx[b0 + m] = __float_as_uint(p.w);
            p.w = __uint_as_float(e - b);
            s[m] = p;
            float4 lo = make_float4(p.x, p.y, p.z, 0.0f), hi = lo;
            if (m > b)
            {
                const uint32_t c = b0 + b + (m - b) / 2;
                const float4 cl = box[2 * c], ch = box[2 * c + 1];
                lo = make_float4(fminf(lo.x, cl.x), fminf(lo.y, cl.y), fminf(lo.z, cl.z), 0.0f);
                hi = make_float4(fmaxf(hi.x, ch.x), fmaxf(hi.y, ch.y), fmaxf(hi.z, ch.z), 0.0f);
            }
            if (m + 1 < e)
            {
                const uint32_t c = b0 + m + 1 + (e - m - 1) / 2;
                const float4 cl = box[2 * c], ch = box[2 * c + 1];
                lo = make_float4(fminf(lo.x, cl.x), fminf(lo.y, cl.y), fminf(lo.z, cl.z), 0.0f);
                hi = make_float4(fmaxf(hi.x, ch.x), fmaxf(hi.y, ch.y), fmaxf(hi.z, ch.z), 0.0f);
            }
            box[2 * (b0 + m)] = lo;
            box[2 * (b0 + m) + 1] = hi;
        }
        __syncthreads();
    }
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
        g[b0 + k] = s[k];
}

// One partition round by a cluster of kKtCluster CTAs on a[first, last) (the median of three into
// a[first] by rank 0, then the same parallel Hoare replay as kt_round_block): every CTA takes a
// slice of [first + 1, last), counts its candidates, learns the counts of the slices before it
// through distributed shared memory and writes its positions in order; rank 0 finds T and the cut;
// the swaps are spread over the whole cluster. Cluster barriers order the global-memory steps.
struct KtClusterShared
{
    uint32_t warp_sum[kKtThreads / 32];
    uint32_t cnt[2]; // this CTA's ge, le counts
    uint32_t res[2]; // rank 0: T, cut
};

__device__ uint32_t block_sum(uint32_t v, uint32_t* warp_sum)
{
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0)
        warp_sum[warp] = v;
    __syncthreads();
    uint32_t t = 0;
    for (uint32_t w = 0; w < nwarps; ++w)
        t += warp_sum[w];
    return t;
}

__device__ uint32_t kt_round_cluster(float4* a, uint32_t first, uint32_t last, int ax, uint32_t* ge, uint32_t* le,
                                     KtClusterShared& sh, cg::cluster_group& cluster)
{
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const uint32_t rank = cluster.block_rank();
    if (rank == 0 && tid == 0)
        kt_median_to_first(a, first, last, ax);
    cluster.sync();
    const float p = kt_coord(a[first], ax);
    const uint32_t lo = first + 1, n = last - lo;
    const uint32_t cs = (n + kKtCluster - 1) / kKtCluster;
    const uint32_t c0 = min(n, rank * cs), c1 = min(n, c0 + cs);
    // pass 1: this slice's counts
    uint32_t cge = 0, cle = 0;
    for (uint32_t k = c0 + tid; k < c1; k += blockDim.x)
    {
        const float v = kt_coord(a[lo + k], ax);
        cge += !(v < p) ? 1u : 0u;
        cle += !(p < v) ? 1u : 0u;
    }
    const uint32_t tge = block_sum(cge, sh.warp_sum);
    const uint32_t tle = block_sum(cle, sh.warp_sum);
    if (tid == 0)
    {
        sh.cnt[0] = tge;
        sh.cnt[1] = tle;
    }
    cluster.sync();
    uint32_t base_ge = 0, base_le = 0, nge = 0, nle = 0;
    for (uint32_t r = 0; r < static_cast<uint32_t>(kKtCluster); ++r)
    {
        const uint32_t* rc = cluster.map_shared_rank(&sh.cnt[0], r);
        const uint32_t g0 = rc[0], l0 = rc[1];
        if (r < rank)
        {
            base_ge += g0;
            base_le += l0;
        }
        nge += g0;
        nle += l0;
    }
    // pass 2: ordered positions of this slice, a tile of blockDim x kKtItems at a time
    const uint32_t tile = blockDim.x * kKtItems;
    uint32_t og_run = base_ge, ol_run = base_le;
    for (uint32_t t0 = c0; t0 < c1; t0 += tile)
    {
        uint32_t fge = 0, fle = 0, ng = 0, nl = 0;
#pragma unroll
        for (int k = 0; k < kKtItems; ++k)
        {
            const uint32_t idx = t0 + tid * kKtItems + k;
            if (idx < c1)
            {
                const float v = kt_coord(a[lo + idx], ax);
                if (!(v < p))
                {
                    fge |= 1u << k;
                    ++ng;
                }
                if (!(p < v))
                {
                    fle |= 1u << k;
                    ++nl;
                }
            }
        }
        const uint32_t pk = ng | (nl << 16);
        uint32_t incl = pk;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= static_cast<uint32_t>(o))
                incl += v;
        }
        __syncthreads();
        if (lane == 31)
            sh.warp_sum[warp] = incl;
        __syncthreads();
        uint32_t wpre = 0, total = 0;
        for (uint32_t w = 0; w < nwarps; ++w)
        {
            const uint32_t v = sh.warp_sum[w];
            if (w < warp)
                wpre += v;
            total += v;
        }
        const uint32_t ex = incl - pk + wpre;
        uint32_t og = og_run + (ex & 0xffffu), ol = ol_run + (ex >> 16);
#pragma unroll
        for (int k = 0; k < kKtItems; ++k)
        {
            const uint32_t pos = lo + t0 + tid * kKtItems + k;
            if (fge & (1u << k))
                ge[og++] = pos;
            if (fle & (1u << k))
                le[ol++] = pos;
        }
        og_run += total & 0xffffu;
        ol_run += total >> 16;
    }
    cluster.sync();
    if (rank == 0 && tid == 0)
    {
        uint32_t lo_t = 0, hi_t = min(nge, nle);
        while (lo_t < hi_t)
        {
            const uint32_t mid = (lo_t + hi_t + 1) / 2;
            if (ge[mid - 1] < le[nle - mid])
                lo_t = mid;
            else
                hi_t = mid - 1;
        }
        const uint32_t T = lo_t;
        sh.res[0] = T;
        sh.res[1] = (T == 0) ? ge[0] : min(T < nge ? ge[T] : 0xffffffffu, le[nle - T]);
    }
    cluster.sync();
    const uint32_t* r0 = cluster.map_shared_rank(&sh.res[0], 0);
    const uint32_t T = r0[0], cut = r0[1];
    const uint32_t nthreads = blockDim.x * kKtCluster;
    for (uint32_t t = rank * blockDim.x + tid; t < T; t += nthreads)
        kt_swap(a, ge[t], le[nle - 1 - t]);
    cluster.sync();
    return cut;
}

// Levels whose ranges exceed kKtHuge: a cluster per range runs the introselect rounds while the
// range is above kKtClusterMin, then its rank 0 finishes it as a single CTA would (a round on one
// CTA reads the range at one SM's share of the bandwidth).
__global__ void __cluster_dims__(kKtCluster, 1, 1) __launch_bounds__(kKtThreads)
    k_kt_level_huge(BatchDev b, int level, uint32_t slots)
{
    extern __shared__ float4 kt_smem[];
    __shared__ KtClusterShared csh;
    __shared__ KtShared sh;
    cg::cluster_group cluster = cg::this_cluster();
    const uint32_t range = blockIdx.x / kKtCluster;
    const uint32_t s = range / slots, j = range % slots;
    if (s >= static_cast<uint32_t>(b.nscan))
        return; // uniform over the cluster
    const ScanDev& sd = b.scans[s];
    uint32_t lb, le;
    if (!kt_range(sd.n_src, level, j, lb, le, nullptr) || le - lb <= kKtHuge)
        return; // uniform over the cluster
    float4* g = b.kt + sd.src_off;
    uint32_t* ge = b.kscr + 2ull * sd.src_off + 2ull * lb;
    uint32_t* lq = ge + (le - lb);
    const uint32_t len = le - lb, nth = lb + len / 2;
    uint32_t first = lb, last = le;
    int depth = 2 * static_cast<int>(floor_log2_u(len));
    while (last - first > kKtClusterMin && depth > 0)
    {
        --depth;
        const uint32_t cut = kt_round_cluster(g, first, last, level % 3, ge, lq, csh, cluster);
        if (cut <= nth)
            first = cut;
        else
            last = cut;
    }
    if (cluster.block_rank() == 0)
    {
        // the rest of the introselect on one CTA
        kt_select_block(g, first, nth, last, depth, level % 3, ge, lq, sh, kt_smem,
                        reinterpret_cast<uint16_t*>(kt_smem + kKtSmall));
        if (threadIdx.x == 0)
        {
            float4 p = g[nth];
            b.kq[sd.src_off + nth] = __float_as_uint(p.w);
            p.w = __uint_as_float(len);
            g[nth] = p;
        }
    }
    cluster.sync(); // no CTA leaves while another may read its shared memory
}

__global__ void k_kt_load(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0)
    {
        b.klo_n[b.nsrc] = 0; // the scanned arrays' last slots (totals after the scans)
        b.kshort[b.nsrc] = 0;
        b.kctr[0] = 0;
    }
    if (i >= b.nsrc)
        return;
    const float4 p = b.src[i];
    // the point's input index rides in .w while the build moves the records (saved in kq when the
    // record becomes a node and .w takes its subtree size)
    b.kt[i] = make_float4(p.x, p.y, p.z, __uint_as_float(i));
}

// One level of the build: CTA (scan, slot j). Ranges above kKtSmall are put in order around their
// middle here; a range of at most kKtSmall whose parent was larger (or the root) builds its whole
// subtree in shared memory.
__global__ void __launch_bounds__(kKtThreads) k_kt_level(BatchDev b, int level, uint32_t slots)
{
    extern __shared__ float4 kt_smem[];
    __shared__ KtShared sh;
    const uint32_t s = blockIdx.x / slots, j = blockIdx.x % slots;
    if (s >= static_cast<uint32_t>(b.nscan))
        return;
    const ScanDev& sd = b.scans[s];
    uint32_t lb, le, plen;
    if (!kt_range(sd.n_src, level, j, lb, le, &plen))
        return;
    float4* g = b.kt + sd.src_off;
    float4* box = b.kbb + 2ull * sd.src_off;
    uint32_t* ge = b.kscr + 2ull * sd.src_off + 2ull * lb;
    uint32_t* lq = ge + (le - lb);
    const uint32_t len = le - lb;
    if (len > kKtHuge)
        return; // k_kt_level_huge
    if (len > kKtSmall)
    {
        const uint32_t nth = lb + len / 2;
        kt_select_block(g, lb, nth, le, 2 * static_cast<int>(floor_log2_u(len)), level % 3, ge, lq, sh, kt_smem,
                        reinterpret_cast<uint16_t*>(kt_smem + kKtSmall));
        if (threadIdx.x == 0)
        {
            float4 p = g[nth];
            b.kq[sd.src_off + nth] = __float_as_uint(p.w);
            p.w = __uint_as_float(len);
            g[nth] = p;
        }
    }
    else if (level == 0 || plen > kKtSmall)
    {
        kt_build_small(g, box, b.kq + sd.src_off, lb, le, level, kt_smem, reinterpret_cast<uint16_t*>(kt_smem + kKtSmall));
    }
}

// Boxes of the nodes above the shared-memory subtrees, one level at a time from the bottom.
__global__ void k_kt_box_level(BatchDev b, int level, uint32_t slots)
{
    const uint64_t t = static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const uint32_t s = static_cast<uint32_t>(t / slots), j = static_cast<uint32_t>(t % slots);
    if (s >= static_cast<uint32_t>(b.nscan))
        return;
    const ScanDev& sd = b.scans[s];
    uint32_t lb, le;
    if (!kt_range(sd.n_src, level, j, lb, le, nullptr) || le - lb <= kKtSmall)
        return;
    const float4* g = b.kt + sd.src_off;
    float4* box = b.kbb + 2ull * sd.src_off;
    const uint32_t m = lb + (le - lb) / 2;
    const float4 p = g[m];
    float4 lo = make_float4(p.x, p.y, p.z, 0.0f), hi = lo;
    const uint32_t cs[2] = {lb + (m - lb) / 2, m + 1 + (le - m - 1) / 2};
    const bool has[2] = {m > lb, m + 1 < le};
    for (int k = 0; k < 2; ++k)
        if (has[k])
        {
            const float4 cl = box[2 * cs[k]], ch = box[2 * cs[k] + 1];
            lo = make_float4(fminf(lo.x, cl.x), fminf(lo.y, cl.y), fminf(lo.z, cl.z), 0.0f);
            hi = make_float4(fmaxf(hi.x, ch.x), fmaxf(hi.y, ch.y), fmaxf(hi.z, ch.z), 0.0f);
        }
    box[2 * m] = lo;
    box[2 * m + 1] = hi;
}

// ---------------------------------------------------------------------------------------------
// The reference's search (kdtree.hpp:355-388) from the entries on stk[0, sp): pop, count the node
// when within r2 (stopping at k), push both children when the splitting plane is within the
// radius (right first, so the left is searched first) or else the side of the query. Empty
// children are not pushed: the reference pushes and pops them without effect. Returns the count;
// after an early stop stk[0, sp) holds the entries left behind.
// ---------------------------------------------------------------------------------------------
__device__ uint32_t kt_search(const float4* __restrict__ g, uint32_t n, float qx, float qy, float qz, float r2,
                              uint32_t k, uint32_t found, uint32_t* stk, int& sp, bool& overflow)
{
    while (sp > 0)
    {
        const uint32_t e = stk[--sp];
        const uint32_t m = e >> 2;
        const int ax = static_cast<int>(e & 3u);
        if (m >= n || ax > 2)
        {
            overflow = true; // not a node of this tree: reported, never followed
            return found;
        }
        const float4 nd = g[m];
        const float d0 = (qx - nd.x) * (qx - nd.x);
        const float d1 = (qy - nd.y) * (qy - nd.y);
        const float d2 = (qz - nd.z) * (qz - nd.z);
        if (d0 + (d1 + d2) <= r2)
        {
            if (++found >= k)
                return found;
        }
        const uint32_t len = __float_as_uint(nd.w);
        if (len == 0 || m < len / 2 || m - len / 2 + len > n)
        {
            overflow = true; // a subtree size the build did not leave: reported, never followed
            return found;
        }
        const uint32_t lb = m - len / 2;
        const uint32_t llen = m - lb, rlen = len - llen - 1;
        const int nx = (ax == 2) ? 0 : ax + 1;
        const float q = (ax == 0) ? qx : ((ax == 1) ? qy : qz);
        const float delta = kt_coord(nd, ax) - q;
        const bool push_r = (delta * delta <= r2) ? true : !(delta > 0);
        const bool push_l = (delta * delta <= r2) ? true : (delta > 0);
        if (sp + 2 > kKtStack)
        {
            overflow = true;
            return found;
        }
        if (push_r && rlen)
            stk[sp++] = kt_entry(m + 1 + rlen / 2, nx);
        if (push_l && llen)
            stk[sp++] = kt_entry(lb + llen / 2, nx);
    }
    return found;
}

// A subtree whose box lies farther than the radius holds no match: the reference's search
// through it ends without counting anything. The box distance is formed in binary32 exactly as
// kt_search forms a point's distance (per-axis difference, square, d0 + (d1 + d2)). Rounding to
// nearest is monotone and odd, so for every point p of the box |fl(q - p)| >= fl(gap) on each axis
// (the gap being the box's bound minus q, or 0 inside the slab), and each square and partial sum of
// p's distance is at least its counterpart here: when this sum exceeds r2, so does p's, and no
// subtree that could hold a match is skipped. (Binary32 keeps the test off the binary64 pipe,
// which runs at a small fraction of the binary32 rate on this GPU.)
__device__ __forceinline__ bool kt_may_hit(const float4* __restrict__ box, uint32_t m, float qx, float qy, float qz,
                                           float r2)
{
    const float4 lo = box[2 * m], hi = box[2 * m + 1];
    auto gap = [](float q, float l, float h) -> float { return (q < l) ? (l - q) : ((q > h) ? (q - h) : 0.0f); };
    const float gx = gap(qx, lo.x, hi.x), gy = gap(qy, lo.y, hi.y), gz = gap(qz, lo.z, hi.z);
    return (gx * gx) + ((gy * gy) + (gz * gz)) <= r2;
}

__device__ __forceinline__ int kt_scan_of(const BatchDev& b, uint32_t i)
{
    return find_scan(b.nscan, i, [&](int s) { return b.scans[s].src_off; });
}

// Pool allocation of `count` entries, one atomic per group of converged lanes (the lanes loop
// over the group's members alike, so every shuffle has all of them); kNone when the pool is full.
__device__ __forceinline__ uint32_t kt_pool_alloc(uint32_t* head, uint32_t cap, uint32_t count)
{
    const uint32_t active = __activemask();
    const uint32_t lane = lane_id();
    uint32_t pre = 0, total = 0;
    for (uint32_t l = 0; l < 32; ++l)
        if ((active >> l) & 1u)
        {
            const uint32_t c = __shfl_sync(active, count, l);
            total += c;
            if (l < lane)
                pre += c;
        }
    const uint32_t leader = static_cast<uint32_t>(__ffs(static_cast<int>(active)) - 1);
    uint32_t base = 0;
    if (lane == leader && total)
        base = atomicAdd(head, total);
    base = __shfl_sync(active, base, leader);
    if (base > cap || cap - base < total)
        return kNone;
    return base + pre;
}

// Step 2: every point's own search; VALID points' leftovers into the pool. Thread t takes the
// point at tree position t (its input index from the build), so the threads of a warp query
// neighbouring points, whose searches walk largely the same nodes (cache hits, little divergence,
// where input order may be shuffled); the results go to the point's input index.
__global__ void k_kt_own(BatchDev b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= b.nsrc)
        return;
    const int s = kt_scan_of(b, t);
    const ScanDev& sd = b.scans[s];
    const float4 q = b.kt[t]; // the point's coordinates, as loaded from the input
    const uint32_t i = b.kq[t];
    if (i - sd.src_off >= sd.n_src)
    {
        raise_err(&b.state[s], ERR_INTERNAL); // not a point of this scan: reported, never followed
        return;
    }
    const float r2 = kt_radius2(sd, q);
    uint32_t stk[kKtStack];
    int sp = 0;
    bool overflow = false;
    stk[sp++] = kt_entry(sd.n_src / 2, 0);
    const float4* g = b.kt + sd.src_off;
    const uint32_t k = sd.dror_k;
    const uint32_t found = kt_search(g, sd.n_src, q.x, q.y, q.z, r2, k, 0, stk, sp, overflow);
    if (overflow)
        raise_err(&b.state[s], ERR_INTERNAL);
    const bool valid = found >= k;
    b.kown[i] = found;
    b.kshort[i] = valid ? 0u : 1u;
    uint32_t nleft = valid ? static_cast<uint32_t>(sp) : 0u;
    const uint32_t at = kt_pool_alloc(b.kctr, b.kpool_cap, nleft);
    if (at == kNone)
    {
        raise_err(&b.state[s], ERR_HASH_FULL); // leftover pool full: reported, scan invalid
        nleft = 0;
    }
    b.klo_n[i] = nleft;
    b.klo_at[i] = (at == kNone) ? 0u : at;
    for (uint32_t t = 0; t < nleft; ++t)
        b.kpool[at + t] = stk[t];
    if (valid)
        b.noise[i] = LP_NOISE_VALID;
}

// Leftovers into one array in point order (klo_off: exclusive scan of the counts).
__global__ void k_kt_flat(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc)
        return;
    const uint32_t n = b.klo_off[i + 1] - b.klo_off[i];
    const uint32_t at = b.klo_at[i], to = b.klo_off[i];
    for (uint32_t t = 0; t < n; ++t)
        b.kflat[to + t] = b.kpool[at + t];
}

// The short points in order (kshort: exclusive scan of the flags).
__global__ void k_kt_short(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc)
        return;
    if (b.kshort[i + 1] != b.kshort[i])
        b.kq[b.kshort[i]] = i;
}

// First entry (flat index) of the piece a short point meets on top of the stack: the leftovers of
// the points after the previous short point of its scan.
// The same for short point u once k_kt_segment has run: it records its piece's first entry in
// klo_n, which holds nothing else by then (one load instead of three dependent ones).
__device__ __forceinline__ uint32_t kt_piece_lo(const BatchDev& b, uint32_t u)
{
    return b.klo_n[u];
}

__device__ __forceinline__ uint32_t kt_segment_lo(const BatchDev& b, const ScanDev& sd, uint32_t t)
{
    const uint32_t first = b.kshort[sd.src_off];
    const uint32_t prev = (t > first) ? b.kq[t - 1] + 1 : sd.src_off;
    return b.klo_off[prev];
}

// Step 3: each short point through its own piece.
__global__ void k_kt_segment(BatchDev b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nshort = b.kshort[b.nsrc];
    if (t >= nshort)
        return;
    const uint32_t i = b.kq[t];
    const int s = kt_scan_of(b, i);
    const ScanDev& sd = b.scans[s];
    const float4 q = b.src[i];
    const float r2 = kt_radius2(sd, q);
    const float4* g = b.kt + sd.src_off;
    const float4* box = b.kbb + 2ull * sd.src_off;
    const uint32_t k = sd.dror_k;
    uint32_t found = b.kown[i];
    const uint32_t lo = kt_segment_lo(b, sd, t), hi = b.klo_off[i];
    b.klo_n[t] = lo; // for the candidate walks and the chain (klo_n is no longer read as counts)
    uint4 res = make_uint4(0u, kNone, 0u, 0u); // found, stop entry, partial leftover at, count
    uint32_t stk[kKtStack];
    bool overflow = false;
    for (uint32_t x = hi; x > lo; --x)
    {
        const uint32_t e = b.kflat[x - 1];
        if (!kt_may_hit(box, e >> 2, q.x, q.y, q.z, r2))
            continue;
        int sp = 0;
        stk[sp++] = e;
        found = kt_search(g, sd.n_src, q.x, q.y, q.z, r2, k, found, stk, sp, overflow);
        if (found >= k)
        {
            uint32_t at = kt_pool_alloc(b.kctr, b.kpool_cap, static_cast<uint32_t>(sp));
            if (at == kNone)
            {
                raise_err(&b.state[s], ERR_HASH_FULL);
                at = 0;
                sp = 0;
            }
            for (int u = 0; u < sp; ++u)
                b.kpool[at + u] = stk[u];
            res = make_uint4(found, x - 1, at, static_cast<uint32_t>(sp));
            b.noise[i] = LP_NOISE_VALID;
            break;
        }
    }
    if (overflow)
        raise_err(&b.state[s], ERR_INTERNAL);
    res.x = found;
    b.kc[t] = res;
}

// Candidates: short points not decided in their own piece (flag -> exclusive scan -> list).
__global__ void k_kt_cand_flag(BatchDev b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nshort = b.kshort[b.nsrc];
    if (t == 0)
        b.kcflag[nshort] = 0;
    if (t < nshort)
        b.kcflag[t] = (b.kc[t].y == kNone) ? 1u : 0u;
}

__global__ void k_kt_cand_list(BatchDev b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < b.kshort[b.nsrc] && b.kcflag[t + 1] != b.kcflag[t])
        b.kcand[b.kcflag[t]] = t;
}

// Walks the pieces the short points (tp, t) of a scan pushed (all decided in their own piece:
// the rest of their piece below the stop, then the entries the stopping search left, on top),
// newest first, for query q from count `found`. Stops where the count reaches k and returns the
// stop: short index u, kind (1: the left entries, 0: the piece rest) and entry index; the entries
// that stopping search left go to the pool.
struct KtStop
{
    uint32_t u, kind, x, at, n;
};

__device__ bool kt_walk_pushed(const BatchDev& b, const ScanDev& sd, const float4* g, const float4* box, uint32_t tp1,
                               uint32_t t, float qx, float qy, float qz, float r2, uint32_t k, uint32_t& found,
                               KtStop& stop, uint32_t* stk, bool& overflow, bool& pool_full)
{
    for (uint32_t u = t; u > tp1;)
    {
        --u;
        const uint4 c = b.kc[u];
        for (int kind = 1; kind >= 0; --kind)
        {
            const uint32_t lo = kind ? c.z : kt_piece_lo(b, u);
            const uint32_t hi = kind ? c.z + c.w : c.y;
            const uint32_t* arr = kind ? b.kpool : b.kflat;
            for (uint32_t x = hi; x > lo; --x)
            {
                const uint32_t e = arr[x - 1];
                if (!kt_may_hit(box, e >> 2, qx, qy, qz, r2))
                    continue;
                int sp = 0;
                stk[sp++] = e;
                found = kt_search(g, sd.n_src, qx, qy, qz, r2, k, found, stk, sp, overflow);
                if (found >= k)
                {
                    uint32_t at = kt_pool_alloc(b.kctr, b.kpool_cap, static_cast<uint32_t>(sp));
                    if (at == kNone)
                    {
                        pool_full = true;
                        at = 0;
                        sp = 0;
                    }
                    for (int v = 0; v < sp; ++v)
                        b.kpool[at + v] = stk[v];
                    stop = KtStop{u, static_cast<uint32_t>(kind), x - 1, at, static_cast<uint32_t>(sp)};
                    return true;
                }
            }
        }
    }
    return false;
}

// Step 4a: every candidate walks the pieces pushed since the previous candidate, as if nothing
// lay below them (true when the previous candidate exhausted the stack).
__global__ void k_kt_spec(BatchDev b)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ncand = b.kcflag[b.kshort[b.nsrc]];
    if (c >= ncand)
        return;
    const uint32_t t = b.kcand[c];
    const uint32_t i = b.kq[t];
    const int s = kt_scan_of(b, i);
    const ScanDev& sd = b.scans[s];
    const uint32_t t_first = b.kshort[sd.src_off];
    const uint32_t c_first = b.kcflag[t_first];
    const uint32_t tp1 = (c > c_first) ? b.kcand[c - 1] + 1 : t_first; // first pushing short point
    const float4 q = b.src[i];
    const float r2 = kt_radius2(sd, q);
    uint32_t found = b.kc[t].x;
    uint32_t stk[kKtStack];
    bool overflow = false, pool_full = false;
    KtStop stop{kNone, 0, 0, 0, 0};
    kt_walk_pushed(b, sd, b.kt + sd.src_off, b.kbb + 2ull * sd.src_off, tp1, t, q.x, q.y, q.z, r2, sd.dror_k, found,
                   stop, stk, overflow, pool_full);
    if (overflow)
        raise_err(&b.state[s], ERR_INTERNAL);
    if (pool_full)
        raise_err(&b.state[s], ERR_HASH_FULL);
    b.kspec[c] = make_uint4(found, stop.u, stop.x | (stop.kind << 31), stop.at);
    b.kspec_n[c] = stop.n;
}

// Record of a candidate's walk through what its predecessor's stop left (k_kt_spec_next), in
// arrays free by then (per candidate c): kscr[2c] stop entry, kscr[2c + 1] where the entries that
// stopping search left start in the pool, kown[c] count, klo_at[c] = status | left count << 2 |
// piece << 9 (the stop's piece, counted from the top of those pieces).
constexpr uint32_t kNextNone = 0u, kNextStop = 1u, kNextOut = 2u;
constexpr uint32_t kNextPieceMax = 1u << 23;

// Step 4a': a candidate whose walk ran out, right after a candidate whose walk stopped, continues
// into R, and R is then what it was before that stop with the stop's pieces on top: the pieces of
// the predecessor's pushing points below its stop point u, the rest of u's pieces below the stop,
// and the entries the stopping search left (the chain pushes exactly these, in this order). Every
// such candidate walks those pieces here, in parallel, from its count after its own walk. The
// chain takes the result when the predecessor's stop is the last change to R: a stop in those
// pieces is exact whatever lies below them; running out of them continues into R below.
__global__ void k_kt_spec_next(BatchDev b)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ncand = b.kcflag[b.kshort[b.nsrc]];
    if (c >= ncand)
        return;
    b.klo_at[c] = kNextNone;
    const uint32_t t = b.kcand[c];
    const uint32_t i = b.kq[t];
    const int s = kt_scan_of(b, i);
    const ScanDev& sd = b.scans[s];
    const uint32_t t_first = b.kshort[sd.src_off];
    const uint32_t c_first = b.kcflag[t_first];
    if (c == c_first)
        return; // the scan's first candidate has no predecessor
    const uint4 own = b.kspec[c], pv = b.kspec[c - 1];
    if (own.y != kNone || pv.y == kNone)
        return; // this walk stopped, or the predecessor's ran out
    const uint32_t tp1 = (c - 1 > c_first) ? b.kcand[c - 2] + 1 : t_first; // the predecessor's first pushing point
    const uint32_t hu = pv.y, hx = pv.z & 0x7fffffffu, hkind = pv.z >> 31;
    const float4 q = b.src[i];
    const float r2 = kt_radius2(sd, q);
    const float4* g = b.kt + sd.src_off;
    const float4* box = b.kbb + 2ull * sd.src_off;
    const uint32_t k = sd.dror_k;
    uint32_t found = own.x;
    uint32_t stk[kKtStack];
    bool overflow = false, pool_full = false;
    uint32_t piece = 0, sx = 0, sat = 0, sn = 0;
    // one piece, entries from hi - 1 down; an empty piece is not in R and is not counted
    auto walk = [&](uint32_t lo, uint32_t hi, bool pool) -> bool {
        if (hi <= lo)
            return false;
        const uint32_t* arr = pool ? b.kpool : b.kflat;
        for (uint32_t x = hi; x > lo; --x)
        {
            const uint32_t e = arr[x - 1];
            if (!kt_may_hit(box, e >> 2, q.x, q.y, q.z, r2))
                continue;
            int sp = 0;
            stk[sp++] = e;
            found = kt_search(g, sd.n_src, q.x, q.y, q.z, r2, k, found, stk, sp, overflow);
            if (found >= k)
            {
                uint32_t at = kt_pool_alloc(b.kctr, b.kpool_cap, static_cast<uint32_t>(sp));
                if (at == kNone)
                {
                    pool_full = true;
                    at = 0;
                    sp = 0;
                }
                for (int v = 0; v < sp; ++v)
                    b.kpool[at + v] = stk[v];
                sx = x - 1;
                sat = at;
                sn = static_cast<uint32_t>(sp);
                return true;
            }
        }
        ++piece;
        return false;
    };
    bool stopped = walk(pv.w, pv.w + b.kspec_n[c - 1], true);
    if (!stopped)
    {
        const uint4 cu = b.kc[hu];
        if (hkind == 1)
            stopped = walk(cu.z, hx, true) || walk(kt_piece_lo(b, hu), cu.y, false);
        else
            stopped = walk(kt_piece_lo(b, hu), hx, false);
    }
    for (uint32_t u = hu; !stopped && u > tp1;)
    {
        --u;
        const uint4 cu = b.kc[u];
        stopped = walk(cu.z, cu.z + cu.w, true) || walk(kt_piece_lo(b, u), cu.y, false);
    }
    if (overflow)
        raise_err(&b.state[s], ERR_INTERNAL);
    if (pool_full)
        raise_err(&b.state[s], ERR_HASH_FULL);
    if (piece >= kNextPieceMax || overflow || pool_full)
        return; // the chain searches R itself
    b.kscr[2ull * c] = sx;
    b.kscr[2ull * c + 1] = sat;
    b.kown[c] = found;
    b.klo_at[c] = (stopped ? kNextStop : kNextOut) | (sn << 2) | (piece << 9);
}

// Step 4b: one CTA per scan applies the candidates' walks in order. R, the stack below the pieces
// pushed since the previous candidate, is a list of pieces (lo, hi): entries [lo, hi) of the flat
// array (bit 31 of lo clear) or of the pool (set), consumed from hi - 1 down. A candidate whose
// walk stopped adds what its walk left on top of R. One whose walk ran out continues into R,
// up to kChainThreads entries at a time across the top kChainPieces pieces: every thread searches
// one entry's subtree in full (these searches, chains of dependent node loads, are the chain's
// cost, so a round is as wide as the CTA), and an ordered prefix of the counts finds the stop;
// running out of R too means NOISE and an empty R. While R is empty, a run of candidates whose
// walks ran out is NOISE as a whole. The candidates' records are staged kChainThreads at a time in
// shared memory. Control flow is uniform: every thread holds the same R top, count and candidate;
// thread 0 writes R and the pool, and a barrier precedes every read of them.
constexpr uint32_t kChainThreads = 256;
constexpr uint32_t kChainPieces = 32;

__global__ void __launch_bounds__(kChainThreads) k_kt_chain(BatchDev b)
{
    __shared__ uint32_t red[kChainThreads / 32];
    __shared__ uint32_t bc[4];
    // the window of candidates [w0, w1): walk record, left-entry count, point, its first pushing
    // short point, query
    __shared__ uint4 w_spec[kChainThreads];
    __shared__ uint32_t w_specn[kChainThreads], w_i[kChainThreads], w_tp1[kChainThreads];
    __shared__ float4 w_q[kChainThreads];
    __shared__ uint4 w_nx[kChainThreads]; // walk through the predecessor's stop pieces (k_kt_spec_next)
    // the top pieces of R for one round (index 0 = the top) and their entry-count prefix
    __shared__ uint2 r_pc[kChainPieces];
    __shared__ uint32_t r_pre[kChainPieces + 1];
    const int s = blockIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    ScanState* st = &b.state[s];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const float4* g = b.kt + sd.src_off;
    const float4* box = b.kbb + 2ull * sd.src_off;
    const uint32_t k = sd.dror_k;
    uint2* R = b.kpiece + 2ull * sd.src_off + 2ull * static_cast<uint32_t>(s);
    const uint32_t cap = 2u * sd.n_src + 2u;
    const uint32_t t_first = b.kshort[sd.src_off], t_end = b.kshort[sd.src_off + sd.n_src];
    const uint32_t c0 = b.kcflag[t_first], c1 = b.kcflag[t_end];
    uint32_t top = 0; // pieces in R (the same in every thread)
    // R's top before the last candidate's stop pushed its pieces, while that stop is the last
    // change to R (kNone otherwise)
    uint32_t mark = kNone;
    bool overflow = false, pool_full = false, full = false;
    uint32_t stk[kKtStack];
    auto push = [&](uint32_t lo, uint32_t hi) {
        if (hi > (lo & 0x7fffffffu))
        {
            if (top < cap)
            {
                if (tid == 0)
                    R[top] = make_uint2(lo, hi);
                ++top;
            }
            else
                full = true;
        }
    };
    // block-wide minimum and inclusive sum (every thread gets the result)
    auto block_min = [&](uint32_t v) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0)
            red[warp] = v;
        __syncthreads();
        uint32_t m = red[0];
        for (uint32_t w = 1; w < nwarps; ++w)
            m = min(m, red[w]);
        __syncthreads();
        return m;
    };
    auto block_incl = [&](uint32_t v, uint32_t& total) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= static_cast<uint32_t>(o))
                v += u;
        }
        if (lane == 31)
            red[warp] = v;
        __syncthreads();
        uint32_t pre = 0;
        total = 0;
        for (uint32_t w = 0; w < nwarps; ++w)
        {
            const uint32_t x = red[w];
            if (w < warp)
                pre += x;
            total += x;
        }
        __syncthreads();
        return v + pre;
    };
    uint32_t c = c0, w0 = c0, w1 = c0;
    while (c < c1)
    {
        if (c >= w1)
        {
            // stage the next window of candidates (one per thread)
            w0 = c;
            w1 = min(c + blockDim.x, c1);
            const uint32_t cc = c + tid;
            if (cc < w1)
            {
                const uint32_t t = b.kcand[cc];
                const uint32_t i = b.kq[t];
                w_spec[tid] = b.kspec[cc];
                w_specn[tid] = b.kspec_n[cc];
                w_i[tid] = i;
                w_tp1[tid] = (cc > c0) ? b.kcand[cc - 1] + 1 : t_first;
                w_q[tid] = b.src[i];
                w_nx[tid] = make_uint4(b.kown[cc], b.kscr[2ull * cc], b.kscr[2ull * cc + 1], b.klo_at[cc]);
            }
            __syncthreads();
        }
        if (top == 0)
        {
            // candidates whose walks ran out with R empty are NOISE, up to the first that stopped
            mark = kNone;
            const uint32_t cc = c + tid;
            const bool live = cc < w1;
            const bool hit = live && w_spec[cc - w0].y != kNone;
            const uint32_t h = min(block_min(hit ? tid : kNone), w1 - c);
            if (live && tid < h)
                b.noise[w_i[cc - w0]] = LP_NOISE_NOISE;
            c += h;
            if (c >= w1)
                continue;
        }
        const uint32_t wc = c - w0;
        const uint4 sp4 = w_spec[wc];
        const uint32_t i = w_i[wc];
        if (sp4.y != kNone)
        {
            // the walk stopped at short point u: R gains the pieces of the pushing points below u,
            // then the rest of u's pieces below the stop, then the entries the stopping search left
            mark = top;
            const uint32_t tp1 = w_tp1[wc];
            const uint32_t hu = sp4.y, hx = sp4.z & 0x7fffffffu, hkind = sp4.z >> 31;
            for (uint32_t u = tp1; u <= hu; ++u)
            {
                const uint4 cu = b.kc[u];
                const uint32_t lo = kt_piece_lo(b, u);
                if (u < hu)
                {
                    push(lo, cu.y);
                    push(cu.z | 0x80000000u, cu.z + cu.w);
                }
                else if (hkind == 1)
                {
                    push(lo, cu.y);
                    push(cu.z | 0x80000000u, hx);
                }
                else
                {
                    push(lo, hx);
                }
            }
            push(sp4.w | 0x80000000u, sp4.w + w_specn[wc]);
            if (tid == 0)
                b.noise[i] = LP_NOISE_VALID;
            ++c;
            __syncthreads(); // thread 0's pieces are read by every thread next
            continue;
        }
        // the walk ran out with R non-empty: continue into R
        const float4 q = w_q[wc];
        const float r2 = kt_radius2(sd, q);
        uint32_t found = sp4.x;
        bool hit = false;
        if (mark != kNone)
        {
            // the previous candidate stopped and nothing changed R since: its stop's pieces lie on
            // top of R, and this candidate's walk through them is done
            const uint4 nx = w_nx[wc];
            const uint32_t status = nx.w & 3u, nsp = (nx.w >> 2) & 127u, p = nx.w >> 9;
            if (status == kNextStop && mark + p < top)
            {
                const uint2 pc = R[top - 1 - p];
                top -= p + 1;
                push(pc.x, nx.y);
                push(nx.z | 0x80000000u, nx.z + nsp);
                found = nx.x;
                hit = true;
            }
            else if (status == kNextOut)
            {
                found = nx.x;
                top = mark; // those pieces are used up; R below them follows
            }
            mark = kNone;
        }
        while (top > 0 && !hit)
        {
            // the top pieces (warp 0) and how many entries of them this round covers
            const uint32_t np = min(top, kChainPieces);
            if (warp == 0)
            {
                const uint2 pc = (lane < np) ? R[top - 1 - lane] : make_uint2(0u, 0u);
                const uint32_t sz = (lane < np) ? pc.y - (pc.x & 0x7fffffffu) : 0u;
                uint32_t incl = sz;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t u = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= static_cast<uint32_t>(o))
                        incl += u;
                }
                if (lane < np)
                    r_pc[lane] = pc;
                r_pre[lane + 1] = incl;
                if (lane == 0)
                    r_pre[0] = 0;
            }
            __syncthreads();
            const uint32_t covered = min(r_pre[np], blockDim.x);
            uint32_t cnt = 0, my_p = 0;
            if (tid < covered)
            {
                // the piece holding this thread's entry: the last p with r_pre[p] <= tid
                uint32_t lo_p = 0, hi_p = np - 1;
                while (lo_p < hi_p)
                {
                    const uint32_t mid = (lo_p + hi_p + 1) / 2;
                    if (r_pre[mid] <= tid)
                        lo_p = mid;
                    else
                        hi_p = mid - 1;
                }
                my_p = lo_p;
                const uint2 pc = r_pc[my_p];
                const uint32_t* arr = (pc.x & 0x80000000u) ? b.kpool : b.kflat;
                const uint32_t e = arr[pc.y - 1 - (tid - r_pre[my_p])];
                if (kt_may_hit(box, e >> 2, q.x, q.y, q.z, r2))
                {
                    int sp = 0;
                    stk[sp++] = e;
                    cnt = kt_search(g, sd.n_src, q.x, q.y, q.z, r2, k, 0, stk, sp, overflow);
                }
            }
            uint32_t total = 0;
            const uint32_t incl = block_incl(cnt, total);
            const bool reach_here = tid < covered && cnt > 0 && found + incl >= k;
            const uint32_t hl = block_min(reach_here ? tid : kNone);
            if (hl != kNone)
            {
                if (tid == hl)
                {
                    bc[0] = found + incl - cnt; // the count before the stopping entry
                    bc[3] = my_p;
                }
                __syncthreads();
                const uint32_t before = bc[0], p = bc[3];
                const uint2 pc = r_pc[p];
                const uint32_t x = pc.y - 1 - (hl - r_pre[p]);
                const uint32_t* arr = (pc.x & 0x80000000u) ? b.kpool : b.kflat;
                // the stopping search again on thread 0, from the count before it, for what it leaves
                if (tid == 0)
                {
                    int sp = 0;
                    stk[sp++] = arr[x];
                    kt_search(g, sd.n_src, q.x, q.y, q.z, r2, k, before, stk, sp, overflow);
                    uint32_t at = kt_pool_alloc(b.kctr, b.kpool_cap, static_cast<uint32_t>(sp));
                    if (at == kNone)
                    {
                        pool_full = true;
                        at = 0;
                        sp = 0;
                    }
                    for (int v = 0; v < sp; ++v)
                        b.kpool[at + v] = stk[v];
                    bc[1] = static_cast<uint32_t>(sp);
                    bc[2] = at;
                }
                __syncthreads();
                const uint32_t nsp = bc[1], at = bc[2];
                // R: the pieces above p are consumed, p keeps its entries below the stop, then the
                // left entries go on top
                top -= p + 1;
                push(pc.x, x);
                push(at | 0x80000000u, at + nsp);
                hit = true;
            }
            else
            {
                found += total;
                // pieces fully covered are consumed; the last covered one keeps what lies below
                uint32_t p = 0;
                while (p < np && r_pre[p + 1] <= covered)
                    ++p;
                top -= p;
                if (p < np && covered > r_pre[p] && tid == 0)
                    R[top - 1].y = r_pc[p].y - (covered - r_pre[p]);
            }
            __syncthreads();
        }
        if (tid == 0)
            b.noise[i] = hit ? LP_NOISE_VALID : LP_NOISE_NOISE;
        ++c;
        __syncthreads();
    }
    if (__syncthreads_or(overflow) && tid == 0)
        raise_err(st, ERR_INTERNAL);
    if (__syncthreads_or(pool_full) && tid == 0)
        raise_err(st, ERR_HASH_FULL);
    if (full && tid == 0)
        raise_err(st, ERR_INTERNAL);
}
} // namespace

size_t kt_build_smem_bytes()
{
    // the subtree's records, then two uint16 candidate lists per point
    return static_cast<size_t>(kKtSmall) * sizeof(float4) + static_cast<size_t>(kKtSmall) * 2 * sizeof(uint16_t);
}

void init_kdtree_attributes()
{
    cudaFuncSetAttribute(k_kt_level, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kt_build_smem_bytes()));
    cudaFuncSetAttribute(k_kt_level_huge, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kt_build_smem_bytes()));
}

void launch_noise(Launcher& L, const BatchDev& b, const BatchHost& hb, const lp_noise_remover_config& cfg)
{
    (void)cfg;
    const uint32_t T = 256;
    uint32_t nmax = 0;
    for (const ScanDev& sd : hb.scans)
        nmax = std::max(nmax, sd.n_src);
    if (nmax == 0)
        return;
    LP_LAUNCH(L, k_kt_load, div_up(b.nsrc, T), T, b);
    // levels until every range of the deepest level is at most kKtSmall (then built in shared memory)
    int levels = 1;
    while ((nmax >> (levels - 1)) > kKtSmall)
        ++levels;
    const uint32_t S = static_cast<uint32_t>(b.nscan);
    for (int l = 0; l < levels; ++l)
    {
        const uint32_t slots = 1u << l;
        if ((nmax >> l) > kKtHuge)
            LP_LAUNCH_SMEM(L, k_kt_level_huge, S * slots * kKtCluster, kKtThreads, kt_build_smem_bytes(), b, l, slots);
        LP_LAUNCH_SMEM(L, k_kt_level, S * slots, kKtThreads, kt_build_smem_bytes(), b, l, slots);
    }
    for (int l = levels - 2; l >= 0; --l)
    {
        const uint32_t slots = 1u << l;
        LP_LAUNCH(L, k_kt_box_level, div_up(S * slots, 128u), 128, b, l, slots);
    }
    LP_LAUNCH(L, k_kt_own, div_up(b.nsrc, 128u), 128, b);
    L.scan(b.klo_n, b.klo_off, b.nsrc + 1);
    L.scan(b.kshort, b.kshort, b.nsrc + 1);
    LP_LAUNCH(L, k_kt_flat, div_up(b.nsrc, T), T, b);
    LP_LAUNCH(L, k_kt_short, div_up(b.nsrc, T), T, b);
    LP_LAUNCH(L, k_kt_segment, div_up(b.nsrc, 128u), 128, b);
    LP_LAUNCH(L, k_kt_cand_flag, div_up(b.nsrc + 1, T), T, b);
    L.scan(b.kcflag, b.kcflag, b.nsrc + 1);
    LP_LAUNCH(L, k_kt_cand_list, div_up(b.nsrc, T), T, b);
    LP_LAUNCH(L, k_kt_spec, div_up(b.nsrc, 128u), 128, b);
    LP_LAUNCH(L, k_kt_spec_next, div_up(b.nsrc, 128u), 128, b);
    LP_LAUNCH(L, k_kt_chain, S, kChainThreads, b);
}
} // namespace lpg
