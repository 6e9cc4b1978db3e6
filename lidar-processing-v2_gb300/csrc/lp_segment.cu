// lp_segment.cu — ground segmentation kernels (ring partition, polar grid, RECM, RANSAC,
// range-image projection, dilation, jump convolution, label population).
//
// Reference: lidar_processing_lib/src/segmenter.cpp (Segmenter::segment and helpers) and
// src/dataloader/src/dataloader.cpp:68-137 (ring partition). Every binary32 expression keeps
// the reference's operation order; the library is compiled with --fmad=false so that no
// multiply-add is contracted.
#include <cfloat>

#include <mutex>
#include <random>

#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_math.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
constexpr float kPiF = 3.14159274101257324219f;       // M_PIf
constexpr float kPi2F = 1.57079637050628662109f;      // M_PI_2f
constexpr float kPi15F = 4.71238899230957031250f;     // 1.5F * M_PIf (dataloader.cpp:108)
constexpr float kTwoPiF = 6.28318548202514648438f;    // 2.0F * M_PIf == (float)(2*M_PI)
constexpr int kRingTile = 1024;
constexpr int kSmallCell = 32;   // sorted in registers by one warp
constexpr int kMediumCell = 256; // sorted in shared memory by one warp
constexpr uint32_t kLargeCellMax = 8192;

__device__ __forceinline__ int scan_of_cell(const BatchDev& b, uint32_t c)
{
    return find_scan(b.nscan, c, [&](int s) { return b.scans[s].cell_off; });
}
__device__ __forceinline__ int scan_of_near(const BatchDev& b, uint32_t g)
{
    return find_scan(b.nscan, g, [&](int s) { return b.scans[s].near_off; });
}
__device__ __forceinline__ int scan_of_pix(const BatchDev& b, uint32_t p)
{
    return find_scan(b.nscan, p, [&](int s) { return b.scans[s].pix_off; });
}
__device__ __forceinline__ int scan_of_row(const BatchDev& b, uint32_t r)
{
    return find_scan(b.nscan, r, [&](int s) { return b.scans[s].row_off; });
}
__device__ __forceinline__ int scan_of_tile(const BatchDev& b, uint32_t t)
{
    return find_scan(b.nscan, t, [&](int s) { return b.scans[s].tile_off; });
}
__device__ __forceinline__ int scan_of_slice(const BatchDev& b, uint32_t t)
{
    return find_scan(b.nscan, t, [&](int s) { return b.scans[s].slice_off; });
}

// ------------------------------------------------------------------------------------------
// Ring partition (dataloader.cpp:68-137): quadrant of the wrapped azimuth, FOURTH->FIRST
// transitions counted by a prefix scan, ring = first_ring - min(first_ring, count).
// ------------------------------------------------------------------------------------------
__global__ void k_quadrant(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.npts)
        return;
    const float4 p = b.pts[i];
    float az = lpm::cr_atan2f(p.y, p.x);
    az = (az < 0) ? (az + kTwoPiF) : az;
    uint8_t q;
    if (az < kPi2F)
        q = 0;
    else if (az < kPiF)
        q = 1;
    else if (az < kPi15F)
        q = 2;
    else
        q = 3;
    b.quad[i] = q;
}

__device__ __forceinline__ uint32_t ring_flag(const BatchDev& b, const ScanDev& sd, uint32_t i)
{
    // point i (global) starts a new ring: FIRST after FOURTH, not the scan's first point
    return (i > sd.pt_off && b.quad[i] == 0 && b.quad[i - 1] == 3) ? 1u : 0u;
}

__global__ void __launch_bounds__(256) k_ring_count(BatchDev b)
{
    const uint32_t t = blockIdx.x;
    const int s = scan_of_tile(b, t);
    const ScanDev& sd = b.scans[s];
    const uint32_t first = sd.pt_off + (t - sd.tile_off) * kRingTile;
    const uint32_t end = sd.pt_off + b.state[s].n_pts;
    uint32_t c = 0;
    for (uint32_t k = threadIdx.x; k < kRingTile; k += blockDim.x)
    {
        const uint32_t i = first + k;
        if (i < end)
            c += ring_flag(b, sd, i);
    }
    c = warp_sum(c);
    __shared__ uint32_t sm[8];
    if (lane_id() == 0)
        sm[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        uint32_t tot = 0;
        for (int w = 0; w < 8; ++w)
            tot += sm[w];
        b.tile_cnt[t] = tot;
    }
}

// tile_cnt holds the exclusive scan of the per-tile counts over the whole batch.
__global__ void __launch_bounds__(256) k_ring_apply(BatchDev b)
{
    __shared__ uint32_t sm[33];
    const uint32_t t = blockIdx.x;
    const int s = scan_of_tile(b, t);
    const ScanDev& sd = b.scans[s];
    const uint32_t first = sd.pt_off + (t - sd.tile_off) * kRingTile;
    const uint32_t end = sd.pt_off + b.state[s].n_pts;
    const uint32_t base = b.tile_cnt[t] - b.tile_cnt[sd.tile_off];
    // 4 consecutive points per thread keep the scan in point order
    const uint32_t i0 = first + threadIdx.x * 4;
    uint32_t f[4];
    uint32_t loc = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        f[k] = (i0 + k < end) ? ring_flag(b, sd, i0 + k) : 0u;
        loc += f[k];
    }
    uint32_t total;
    uint32_t pre = block_excl_scan(loc, sm, &total) + base;
    const uint32_t fr = static_cast<uint32_t>(sd.first_ring);
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        pre += f[k];
        if (i0 + k < end)
            b.ring[i0 + k] = static_cast<uint16_t>(fr - min(fr, pre));
    }
}

// ------------------------------------------------------------------------------------------
// Polar grid (constructPolarGrid, segmenter.cpp:103-204).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int32_t bin_point(const BatchDev& b, uint32_t i, const float4 p)
{
    const int s = scan_of_point(b, i);
    const ScanDev& sd = b.scans[s];
    if (i - sd.pt_off >= b.state[s].n_pts)
        return -1; // slot left empty by noise removal
    if (p.z < sd.zmin_adj || p.z > sd.zmax_adj)
        return -1;
    const float d = sqrtf(p.x * p.x + p.y * p.y);
    const int32_t radial = static_cast<int32_t>(d / sd.spacing);
    if (d < sd.min_d || d > sd.max_d || radial >= sd.nrad)
        return -1;
    float az = lpm::atan2_approx(p.y, p.x);
    az = (az < 0) ? (az + kTwoPiF) : az;
    const int32_t slice = min(static_cast<int32_t>(az / sd.slice_res), sd.nslice - 1);
    int32_t h;
    if (sd.use_ring)
    {
        h = b.ring[i];
        if (h >= sd.H)
            return -1;
    }
    else
    {
        const float el = lpm::cr_atanf(p.z / d);
        h = static_cast<int32_t>((el - sd.down_rad) / sd.rad_per_px);
        if (h < 0 || h >= sd.H)
            return -1;
    }
    const int32_t w = static_cast<int32_t>(static_cast<uint16_t>(static_cast<float>(sd.W - 1) * az / kTwoPiF));
    b.pt_pix[i] = h * sd.W + w;
    return static_cast<int32_t>(sd.cell_off + static_cast<uint32_t>(slice * sd.nrad + radial));
}

// Two points per thread (i and i + blockDim.x), both loaded before either is binned. Each
// aggregated slot increment covers 32 consecutive points of one warp: a cell's slots come in
// index runs of one 32-point window each (the near-cell ordering relies on it, and checks it).
__global__ void k_bin(BatchDev b)
{
    const uint32_t i0 = blockIdx.x * blockDim.x * 2u + threadIdx.x;
    const uint32_t i1 = i0 + blockDim.x;
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 p0 = (i0 < b.npts) ? b.pts[i0] : z4;
    const float4 p1 = (i1 < b.npts) ? b.pts[i1] : z4;
    const int32_t c0 = (i0 < b.npts) ? bin_point(b, i0, p0) : -1;
    const int32_t c1 = (i1 < b.npts) ? bin_point(b, i1, p1) : -1;
    if (i0 < b.npts)
        b.pt_cell[i0] = c0;
    if (i1 < b.npts)
        b.pt_cell[i1] = c1;
    // slot of the point in its cell (the order within a cell is free: near cells are ordered later)
    const uint32_t s0 = warp_aggregated_inc(b.cell_cnt, static_cast<uint32_t>(c0), c0 >= 0);
    const uint32_t s1 = warp_aggregated_inc(b.cell_cnt, static_cast<uint32_t>(c1), c1 >= 0);
    if (c0 >= 0)
        b.pt_slot[i0] = s0;
    if (c1 >= 0)
        b.pt_slot[i1] = s1;
}

// (the per-point loads are issued before the scan lookup and the branch, which they do not need)
__global__ void k_scatter(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.npts)
        return;
    const int32_t c = b.pt_cell[i];
    const uint32_t slot = b.pt_slot[i];
    const float z = b.pts[i].z;
    if (c < 0)
        return;
    const int s = scan_of_point(b, i);
    const uint32_t pos = b.cell_start[c] + slot;
    b.csr_idx[pos] = static_cast<int32_t>(i - b.scans[s].pt_off);
    b.csr_z[pos] = z;
}

// zlow of a cell (segmenter.cpp:249-260): with the cell's heights sorted, z[k] for the largest k
// in [1, n/2] with z[k] - z[k-1] > 0.5, else z[0].
//
// No sort is needed for it. Heights fall into half-metre buckets [q/2, (q+1)/2) with
// q = floor(2z) (2z and floor are exact in binary32). Two heights of one bucket differ by less
// than 0.5, so their float difference is at most 0.5: a qualifying k can only be where the sorted
// order crosses from a non-empty bucket A to the next non-empty bucket B, with z[k] = min(B),
// z[k-1] = max(A) and k = the number of heights below B. A warp therefore accumulates count, min
// and max per bucket and evaluates exactly the reference's test at those boundaries. Cells whose
// heights leave the bucket range (a nan, a range over 16 m) take the sorting path.
__device__ __forceinline__ uint32_t zord(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float zunord(uint32_t u)
{
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

__device__ __forceinline__ bool cell_zlow_hist(const BatchDev& b, const ScanDev& sd, uint32_t c, uint32_t n, uint32_t start)
{
    const uint32_t lane = lane_id();
    const int32_t q0 = static_cast<int32_t>(floorf(2.0f * sd.zmin_adj));
    const int32_t nb = static_cast<int32_t>(floorf(2.0f * sd.zmax_adj)) - q0 + 1;
    if (!(nb >= 1 && nb <= 32))
        return false;
    // lane q accumulates bucket q; each step of 32 heights is folded in once per distinct bucket
    // (ground cells hold one or two) with warp reductions instead of contended atomics
    uint32_t cnt = 0u, lo = 0xffffffffu, hi = 0u;
    bool bad = false;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t k = base + lane;
        int32_t q = -1;
        uint32_t zo = 0u;
        if (k < n)
        {
            const float z = b.csr_z[start + k];
            const float f = floorf(2.0f * z);
            if (f >= static_cast<float>(q0) && f < static_cast<float>(q0 + nb))
            {
                q = static_cast<int32_t>(f) - q0;
                zo = zord(z);
            }
            else
                bad = true; // nan or outside the bucket range
        }
        uint32_t todo = __ballot_sync(0xffffffffu, q >= 0);
        while (todo)
        {
            const int32_t lq = __shfl_sync(0xffffffffu, q, __ffs(todo) - 1);
            const bool mine = q == lq;
            const uint32_t gm = __ballot_sync(0xffffffffu, mine);
            const uint32_t glo = __reduce_min_sync(0xffffffffu, mine ? zo : 0xffffffffu);
            const uint32_t ghi = __reduce_max_sync(0xffffffffu, mine ? zo : 0u);
            if (lane == static_cast<uint32_t>(lq))
            {
                cnt += static_cast<uint32_t>(__popc(gm));
                lo = min(lo, glo);
                hi = max(hi, ghi);
            }
            todo &= ~gm;
        }
    }
    if (__any_sync(0xffffffffu, bad))
        return false;
    // lane q = bucket q: position of its first height, previous non-empty bucket
    const uint32_t below = warp_incl_scan(cnt) - cnt;
    int32_t last = (cnt > 0u) ? static_cast<int32_t>(lane) : -1; // inclusive max-scan of non-empty
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int32_t t = __shfl_up_sync(0xffffffffu, last, o);
        if (lane >= static_cast<uint32_t>(o))
            last = max(last, t);
    }
    int32_t prev = __shfl_up_sync(0xffffffffu, last, 1);
    if (lane == 0)
        prev = -1;
    const uint32_t hprev = __shfl_sync(0xffffffffu, hi, max(prev, 0));
    bool qual = false;
    if (cnt > 0u && prev >= 0 && below <= n / 2)
        qual = (zunord(lo) - zunord(hprev)) > 0.5F;
    const uint32_t qm = __ballot_sync(0xffffffffu, qual);
    const uint32_t ne = __ballot_sync(0xffffffffu, cnt > 0u);
    const int32_t pick = qm ? (31 - __clz(qm)) : (__ffs(ne) - 1); // no boundary: z[0], the lowest bucket
    const uint32_t zpick = __shfl_sync(0xffffffffu, lo, pick);
    if (lane == 0)
        b.zlow[c] = zunord(zpick);
    return true;
}

// Fallback for a cell the buckets cannot take (at most kMediumCell heights): warp bitonic sort.
__device__ __forceinline__ void cell_zlow_sorted(const BatchDev& b, uint32_t c, uint32_t n, uint32_t start, float* zs)
{
    const uint32_t lane = lane_id();
    const uint32_t np2 = next_pow2(n);
    for (uint32_t k = lane; k < np2; k += 32)
        zs[k] = (k < n) ? b.csr_z[start + k] : INFINITY;
    __syncwarp();
    warp_bitonic_smem(zs, np2, [](float a, float bb) { return a < bb; });
    int kbest = 0;
    for (uint32_t k = 1 + lane; k <= n / 2; k += 32)
        if (zs[k] - zs[k - 1] > 0.5F)
            kbest = static_cast<int>(k); // lanes visit k in increasing order
    kbest = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(kbest)));
    if (lane == 0)
        b.zlow[c] = zs[kbest];
    __syncwarp();
}

// large_list entries: the cell, bit 31 set when its zlow still has to be found by sorting.
constexpr uint32_t kLargeNeedsZ = 0x80000000u;

// Per-warp scratch of the near-cell ordering: run starts and run destinations.
struct RunScratch
{
    uint16_t rs[kMediumCell + 1];
    uint16_t rd[kMediumCell];
};

// Puts the indices of a near cell (32 < n <= kMediumCell) in ascending order, as the reference's
// cell vectors hold them (segmenter.cpp:99-131 appends in cloud order).
//
// k_bin hands each warp's points of a cell one contiguous slot range in lane order, and a warp
// covers 32 consecutive indices, so a cell's list is a few ascending runs (one per contributing
// warp) over disjoint index ranges. The list is split into runs at every descent and at every
// change of 32-index window (`wofs` = the scan's first batch index mod 32 aligns the windows with
// the warps), the runs are ordered by their first index (a sort of r keys instead of n), and every
// run moves as a block. The result is checked: when one run's last index is not below the next
// run's first, the ranges overlap and the whole list is sorted instead. `is` holds n rounded up
// to a power of two entries, `key` as many. The heights cz (csr_z) are permuted alongside.
__device__ __forceinline__ void warp_order_near(int32_t* csr, float* cz, const float4* pts, uint32_t n, uint32_t wofs,
                                                int32_t* is, float* zb, uint32_t* key, RunScratch& rsc)
{
    const uint32_t lane = lane_id();
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t r = 0;
    int32_t prev = 0, vmin = INT32_MAX, vmax = INT32_MIN;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t k = base + lane;
        const int32_t v = (k < n) ? csr[k] : INT32_MAX;
        is[k] = v;
        zb[k] = (k < n) ? cz[k] : 0.0F;
        int32_t up = __shfl_up_sync(0xffffffffu, v, 1);
        if (lane == 0)
            up = prev;
        const bool head = (k < n) && (k == 0 || v <= up || ((v + wofs) >> 5) != ((up + wofs) >> 5));
        const uint32_t hm = __ballot_sync(0xffffffffu, head);
        if (head)
            rsc.rs[r + __popc(hm & lt)] = static_cast<uint16_t>(k);
        r += __popc(hm);
        prev = __shfl_sync(0xffffffffu, v, 31);
        if (k < n)
        {
            vmin = min(vmin, v);
            vmax = max(vmax, v);
        }
    }
    if (r == 1)
        return; // already ascending
    vmin = __reduce_min_sync(0xffffffffu, vmin);
    vmax = __reduce_max_sync(0xffffffffu, vmax);
    if (lane == 0)
        rsc.rs[r] = static_cast<uint16_t>(n);
    __syncwarp();
    const uint32_t np2 = next_pow2(n);
    // run keys: first index relative to the cell's smallest (24 bits), run id (8 bits)
    bool ok = static_cast<uint32_t>(vmax - vmin) < (1u << 24);
    if (ok && r <= 32)
    {
        uint32_t kv = UINT32_MAX;
        if (lane < r)
            kv = (static_cast<uint32_t>(is[rsc.rs[lane]] - vmin) << 8) | lane;
        kv = warp_bitonic_sort(kv, [](uint32_t a, uint32_t bb) { return a < bb; });
        const uint32_t rid = kv & 0xffu;
        const bool live = lane < r;
        const uint32_t len = live ? static_cast<uint32_t>(rsc.rs[rid + 1] - rsc.rs[rid]) : 0u;
        const int32_t last = live ? is[rsc.rs[rid + 1] - 1] : INT32_MIN;
        const int32_t nhead = live ? is[rsc.rs[rid]] : INT32_MAX;
        const int32_t nxt = __shfl_down_sync(0xffffffffu, nhead, 1);
        ok = __all_sync(0xffffffffu, lane + 1 >= r || last < nxt);
        uint32_t dst = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t t = __shfl_up_sync(0xffffffffu, dst, o);
            if (lane >= static_cast<uint32_t>(o))
                dst += t;
        }
        if (ok && live)
            rsc.rd[rid] = static_cast<uint16_t>(dst - len);
    }
    else if (ok)
    {
        const uint32_t rp2 = next_pow2(r);
        for (uint32_t j = lane; j < rp2; j += 32)
            key[j] = (j < r) ? ((static_cast<uint32_t>(is[rsc.rs[j]] - vmin) << 8) | j) : UINT32_MAX;
        __syncwarp();
        warp_bitonic_smem(key, rp2, [](uint32_t a, uint32_t bb) { return a < bb; });
        uint32_t carry = 0;
        bool good = true;
        for (uint32_t base = 0; base < r; base += 32)
        {
            const uint32_t p = base + lane;
            const bool live = p < r;
            const uint32_t rid = live ? (key[p] & 0xffu) : 0u;
            const uint32_t len = live ? static_cast<uint32_t>(rsc.rs[rid + 1] - rsc.rs[rid]) : 0u;
            if (live && p + 1 < r)
                good &= is[rsc.rs[rid + 1] - 1] < is[rsc.rs[key[p + 1] & 0xffu]];
            uint32_t dst = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t t = __shfl_up_sync(0xffffffffu, dst, o);
                if (lane >= static_cast<uint32_t>(o))
                    dst += t;
            }
            if (live)
                rsc.rd[rid] = static_cast<uint16_t>(carry + dst - len);
            carry += __shfl_sync(0xffffffffu, dst, 31);
        }
        ok = __all_sync(0xffffffffu, good);
    }
    __syncwarp();
    if (!ok)
    {
        for (uint32_t k = ((n + 31u) & ~31u) + lane; k < np2; k += 32)
            is[k] = INT32_MAX;
        __syncwarp();
        warp_bitonic_smem(is, np2, [](int32_t a, int32_t bb) { return a < bb; });
        for (uint32_t k = lane; k < n; k += 32)
        {
            csr[k] = is[k];
            cz[k] = pts[is[k]].z; // the height follows its index
        }
        __syncwarp();
        return;
    }
    uint32_t seen = 0;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t k = base + lane;
        const bool head = (k < n) && (k == 0 || is[k] <= is[k - 1] || ((is[k] + wofs) >> 5) != ((is[k - 1] + wofs) >> 5));
        const uint32_t hm = __ballot_sync(0xffffffffu, head);
        if (k < n)
        {
            const uint32_t rid = seen + __popc(hm & (lt | (1u << lane))) - 1u;
            const uint32_t dst = rsc.rd[rid] + (k - rsc.rs[rid]);
            csr[dst] = is[k];
            cz[dst] = zb[k];
        }
        seen += __popc(hm);
    }
    __syncwarp();
}

__device__ __forceinline__ void cell_small_one(const BatchDev& b, uint32_t c, uint32_t n, uint32_t start, float* zs,
                                               int32_t* is, float* zb, RunScratch& rsc)
{
    const uint32_t lane = lane_id();
    const int s = scan_of_cell(b, c);
    const ScanDev& sd = b.scans[s];
    const bool near = static_cast<int32_t>((c - sd.cell_off) % static_cast<uint32_t>(sd.nrad)) < kRansacRadialBins;
    bool need_z = !cell_zlow_hist(b, sd, c, n, start);
    if (need_z && n <= static_cast<uint32_t>(kMediumCell))
    {
        cell_zlow_sorted(b, c, n, start, zs);
        need_z = false;
    }
    // the RANSAC candidates of a near cell are read in cloud order: sort its indices
    if (need_z || (near && n > static_cast<uint32_t>(kMediumCell)))
    {
        if (lane == 0)
        {
            const uint32_t k = atomicAdd(b.n_large, 1u);
            b.large_list[k] = c | (need_z ? kLargeNeedsZ : 0u);
        }
        return;
    }
    if (!near)
        return;
    if (n > kSmallCell)
    {
        warp_order_near(b.csr_idx + start, b.csr_z + start, b.pts + sd.pt_off, n, sd.pt_off & 31u, is, zb,
                        reinterpret_cast<uint32_t*>(zs), rsc);
        return;
    }
    // (index, height) pairs sorted by index in registers
    int32_t idx = (lane < n) ? b.csr_idx[start + lane] : INT32_MAX;
    float zv = (lane < n) ? b.csr_z[start + lane] : 0.0F;
#pragma unroll
    for (uint32_t k = 2; k <= 32; k <<= 1)
    {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            const int32_t oi = __shfl_xor_sync(0xffffffffu, idx, j);
            const float oz = __shfl_xor_sync(0xffffffffu, zv, j);
            const bool up = ((lane & k) == 0), lower = ((lane & j) == 0);
            if ((lower == up) ? (oi < idx) : (idx < oi))
            {
                idx = oi;
                zv = oz;
            }
        }
    }
    if (lane < n)
    {
        b.csr_idx[start + lane] = idx;
        b.csr_z[start + lane] = zv;
    }
}

__global__ void __launch_bounds__(256) k_cell_small(BatchDev b)
{
    __shared__ float wz[8][kMediumCell];
    __shared__ int32_t wi[8][kMediumCell];
    __shared__ RunScratch wr[8];
    __shared__ float wzb[8][kMediumCell];
    const uint32_t warp = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    // 32 consecutive cells per warp step: one coalesced read of their counts, then only the
    // occupied ones are visited (most cells of a scan are empty)
    for (uint32_t c0 = (blockIdx.x * (blockDim.x >> 5) + warp) * 32u; c0 < b.ncell; c0 += nwarps * 32u)
    {
        const uint32_t c = c0 + lane;
        const uint32_t cnt = (c < b.ncell) ? b.cell_cnt[c] : 0u;
        const uint32_t st = (cnt != 0u) ? b.cell_start[c] : 0u;
        uint32_t m = __ballot_sync(0xffffffffu, cnt != 0u);
        while (m)
        {
            const int j = __ffs(m) - 1;
            m &= m - 1u;
            cell_small_one(b, c0 + static_cast<uint32_t>(j), __shfl_sync(0xffffffffu, cnt, j),
                           __shfl_sync(0xffffffffu, st, j), wz[warp], wi[warp], wzb[warp], wr[warp]);
        }
    }
}

__global__ void __launch_bounds__(512) k_cell_large(BatchDev b)
{
    __shared__ float sz[kLargeCellMax];
    __shared__ int32_t sk;
    const uint32_t nl = *b.n_large;
    for (uint32_t li = blockIdx.x; li < nl; li += gridDim.x)
    {
        const uint32_t entry = b.large_list[li];
        const uint32_t c = entry & ~kLargeNeedsZ;
        const bool need_z = (entry & kLargeNeedsZ) != 0u;
        const uint32_t n = b.cell_cnt[c];
        const uint32_t start = b.cell_start[c];
        const int s = scan_of_cell(b, c);
        const ScanDev& sd = b.scans[s];
        if (n > kLargeCellMax)
        {
            if (threadIdx.x == 0)
            {
                raise_err(&b.state[s], ERR_CELL_TOO_LARGE);
                if (need_z)
                    b.zlow[c] = b.csr_z[start];
            }
            continue;
        }
        const uint32_t np2 = next_pow2(n);
        if (need_z)
        {
            for (uint32_t k = threadIdx.x; k < np2; k += blockDim.x)
                sz[k] = (k < n) ? b.csr_z[start + k] : INFINITY;
            if (threadIdx.x == 0)
                sk = 0;
            __syncthreads();
            block_bitonic_sort(sz, np2, [](float a, float bb) { return a < bb; });
            for (uint32_t k = 1 + threadIdx.x; k <= n / 2; k += blockDim.x)
                if (sz[k] - sz[k - 1] > 0.5F)
                    atomicMax(&sk, static_cast<int32_t>(k));
            __syncthreads();
            if (threadIdx.x == 0)
                b.zlow[c] = sz[sk];
            __syncthreads();
        }
        const bool near = static_cast<int32_t>((c - sd.cell_off) % static_cast<uint32_t>(sd.nrad)) < kRansacRadialBins;
        if (near)
        {
            int32_t* si = reinterpret_cast<int32_t*>(sz);
            for (uint32_t k = threadIdx.x; k < np2; k += blockDim.x)
                si[k] = (k < n) ? b.csr_idx[start + k] : INT32_MAX;
            __syncthreads();
            block_bitonic_sort(si, np2, [](int32_t a, int32_t bb) { return a < bb; });
            for (uint32_t k = threadIdx.x; k < n; k += blockDim.x)
            {
                b.csr_idx[start + k] = si[k];
                b.csr_z[start + k] = b.pts[sd.pt_off + static_cast<uint32_t>(si[k])].z; // the height follows its index
            }
        }
        __syncthreads();
    }
}

// RECM elevation chain per azimuth slice (segmenter.cpp:215-267).
__global__ void k_chain(BatchDev b, uint32_t nslices_total)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= nslices_total)
        return;
    const int s = scan_of_slice(b, g);
    const ScanDev& sd = b.scans[s];
    const uint32_t slice = g - sd.slice_off;
    const uint32_t off = sd.cell_off + slice * static_cast<uint32_t>(sd.nrad);
    float prev = -sd.sensor_h + sd.thr;
    b.elev[off] = prev;
    // the cells' counts and lowest heights do not depend on the chain: 16 cells are loaded before
    // their links are computed (the loads cannot pass the stores to elev otherwise)
    constexpr int32_t kAhead = 16;
    for (int32_t r0 = 1; r0 < sd.nrad; r0 += kAhead)
    {
        uint32_t cnt[kAhead];
        float zlo[kAhead];
#pragma unroll
        for (int32_t u = 0; u < kAhead; ++u)
        {
            const int32_t r = r0 + u;
            cnt[u] = 0u;
            zlo[u] = 0.0f;
            if (r < sd.nrad)
            {
                const uint32_t c = off + static_cast<uint32_t>(r);
                cnt[u] = b.cell_cnt[c];
                zlo[u] = b.zlow[c];
            }
        }
#pragma unroll
        for (int32_t u = 0; u < kAhead; ++u)
        {
            const int32_t r = r0 + u;
            if (r < sd.nrad)
            {
                float e;
                if (cnt[u] == 0)
                {
                    e = prev + sd.delta;
                }
                else
                {
                    const float lim = prev + sd.delta;
                    e = (lim < zlo[u]) ? lim : zlo[u]; // std::min(curr_z_min, prev + delta)
                }
                b.elev[off + static_cast<uint32_t>(r)] = e;
                prev = e;
            }
        }
    }
}

// ------------------------------------------------------------------------------------------
// RANSAC near-field correction (correctCloseRangeFalsePositivesRANSAC, segmenter.cpp:321-479).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t near_cell(const ScanDev& sd, uint32_t k)
{
    const uint32_t slice = k / static_cast<uint32_t>(sd.nnear_per_slice);
    const uint32_t radial = k % static_cast<uint32_t>(sd.nnear_per_slice);
    return sd.cell_off + slice * static_cast<uint32_t>(sd.nrad) + radial;
}

__global__ void __launch_bounds__(256) k_near(BatchDev b, int write)
{
    const uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (g >= b.nnear)
        return;
    const uint32_t lane = lane_id();
    const int s = scan_of_near(b, g);
    const ScanDev& sd = b.scans[s];
    const uint32_t c = near_cell(sd, g - sd.near_off);
    const uint32_t n = b.cell_cnt[c];
    const uint32_t start = b.cell_start[c];
    const float e = b.elev[c];
    const float lim = 2.0F * sd.thr;
    uint32_t pos = write ? b.near_start[g] : 0u;
    for (uint32_t base = 0; base < n; base += 32)
    {
        const uint32_t k = base + lane;
        // csr_z holds the near cells' heights in index order (permuted with csr_idx)
        const bool pred = k < n && fabsf(e - b.csr_z[start + k]) < lim;
        const uint32_t m = __ballot_sync(0xffffffffu, pred);
        if (write && pred)
        {
            const float4 p = b.pts[sd.pt_off + static_cast<uint32_t>(b.csr_idx[start + k])];
            b.cand[pos + __popc(m & ((1u << lane) - 1u))] = make_float4(p.x, p.y, p.z, 0.0f);
        }
        pos += __popc(m);
    }
    if (!write && lane == 0)
        b.near_cnt[g] = pos;
}

// MT19937 (Matsumoto & Nishimura, 1998) and Lemire's nearly divisionless bounded draw
// (Lemire, "Fast Random Integer Generation in an Interval", 2019), which is how
// std::uniform_int_distribution<uint32_t> maps a 32-bit engine onto [0, n-1].
struct Mt19937
{
    uint32_t mt[624];
    int idx;
    __device__ void seed(uint32_t s)
    {
        mt[0] = s;
        for (int i = 1; i < 624; ++i)
            mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + static_cast<uint32_t>(i);
        idx = 624;
    }
    __device__ void twist()
    {
        for (int i = 0; i < 624; ++i)
        {
            const uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
            mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        idx = 0;
    }
    __device__ uint32_t next()
    {
        if (idx >= 624)
            twist();
        uint32_t y = mt[idx++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        return y;
    }
};

// Every scan draws from MT19937 seeded with 42 (segmenter.cpp:328), so its first outputs are the
// same for all scans: they are computed once per device on the host (std::mt19937) and read from
// this table; a scan that needs more (many redraws) runs the generator itself past the table.
constexpr int kMtTable = 4 * 624;
static_assert(kMtTable % 4 == 0, "copied as 16-byte words");
__device__ __align__(16) uint32_t g_mt42[kMtTable];

struct Mt42Stream
{
    const uint32_t* table; // the first kMtTable outputs (a shared-memory copy of g_mt42)
    Mt19937 gen;           // seeded only past the table
    int idx = 0;
    __device__ uint32_t next()
    {
        if (idx < kMtTable)
            return table[idx++];
        if (idx == kMtTable)
        {
            gen.seed(42u);
            for (int k = 0; k < kMtTable; ++k)
                gen.next();
        }
        ++idx;
        return gen.next();
    }
    __device__ uint32_t bounded(uint32_t range) // uniform in [0, range)
    {
        uint64_t m = static_cast<uint64_t>(next()) * range;
        uint32_t l = static_cast<uint32_t>(m);
        if (l < range)
        {
            const uint32_t t = (0u - range) % range;
            while (l < t)
            {
                m = static_cast<uint64_t>(next()) * range;
                l = static_cast<uint32_t>(m);
            }
        }
        return static_cast<uint32_t>(m >> 32);
    }
};

// One warp per scan: lane 0 walks the seed-42 stream (the draws are sequential: a rejected draw
// shifts every later one) and records the index pairs; the lanes then fit the planes in parallel.
__global__ void __launch_bounds__(32) k_ransac_draw(BatchDev b)
{
    __shared__ uint32_t di2[kMaxRansacIters], di3[kMaxRansacIters];
    __shared__ __align__(16) uint32_t mt_table[kMtTable]; // lane 0 walks the stream: shared-memory latency per draw
    __shared__ int bad;
    const int s = blockIdx.x;
    const uint32_t lane = lane_id();
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    const uint32_t first = b.near_start[sd.near_off];
    const uint32_t nnear_s = static_cast<uint32_t>(sd.nslice * sd.nnear_per_slice);
    const uint32_t last = b.near_start[sd.near_off + nnear_s]; // near_start has nnear + 1 entries
    const uint32_t N = last - first;
    if (lane == 0)
    {
        st.cand_off = first;
        st.n_cand = N;
        st.ransac_ok = 0;
        b.pvalid[s] = 0ull;
    }
    if (N < 2)
        return; // the reference never ends its p3 draw for N == 1 (segmenter.cpp:382-386)
    {
        // 16-byte words, several loads in flight per lane
        const uint4* src = reinterpret_cast<const uint4*>(g_mt42);
        uint4* dst = reinterpret_cast<uint4*>(mt_table);
#pragma unroll 5
        for (int k = static_cast<int>(lane); k < kMtTable / 4; k += 32)
            dst[k] = src[k];
    }
    __syncwarp();
    if (lane == 0)
    {
        Mt42Stream gen;
        gen.table = mt_table;
        bad = 0;
        for (int it = 0; it < kMaxRansacIters; ++it)
        {
            const uint32_t i2 = gen.bounded(N);
            uint32_t i3 = gen.bounded(N);
            int guard = 0;
            while (i3 == i2 && guard < (1 << 20))
            {
                i3 = gen.bounded(N);
                ++guard;
            }
            if (guard >= (1 << 20))
            {
                bad = 1;
                break;
            }
            di2[it] = i2;
            di3[it] = i3;
        }
    }
    __syncwarp();
    if (bad)
    {
        if (lane == 0)
            raise_err(&st, ERR_INTERNAL);
        return;
    }
    const float p1x = 0.0F, p1y = 0.0F, p1z = -sd.sensor_h;
    unsigned long long valid = 0ull;
    for (int base = 0; base < kMaxRansacIters; base += 32)
    {
        const int it = base + static_cast<int>(lane);
        bool ok = false;
        if (it < kMaxRansacIters)
        {
            const float4 p2 = b.cand[first + di2[it]];
            const float4 p3 = b.cand[first + di3[it]];
            float nx = ((p2.y - p1y) * (p3.z - p1z)) - ((p2.z - p1z) * (p3.y - p1y));
            float ny = ((p2.z - p1z) * (p3.x - p1x)) - ((p2.x - p1x) * (p3.z - p1z));
            float nz = ((p2.x - p1x) * (p3.y - p1y)) - ((p2.y - p1y) * (p3.x - p1x));
            const float den = (nx * nx) + (ny * ny) + (nz * nz);
            float4 pl = make_float4(0, 0, 0, 0);
            if (!(den < 1.0e-5F))
            {
                const float norm = 1.0F / sqrtf(den);
                nz *= norm;
                if (!(fabsf(nz) < sd.max_cos))
                {
                    nx *= norm;
                    ny *= norm;
                    const float pd = (nx * p1x) + (ny * p1y) + (nz * p1z);
                    pl = make_float4(nx, ny, nz, pd);
                    ok = true;
                }
            }
            b.planes[s * kMaxRansacIters + it] = pl;
            b.inliers[s * kMaxRansacIters + it] = 0u;
        }
        valid |= static_cast<unsigned long long>(__ballot_sync(0xffffffffu, ok)) << base;
    }
    if (lane == 0)
        b.pvalid[s] = valid;
}

// Inlier counts of every hypothesis plane of a scan (segmenter.cpp:409-430): lane l of every
// warp holds planes l and l + 32 as a float pair and counts, for the candidates its warp takes,
// |((n.x p.x + n.y p.y) + n.z p.z) - d| < thr with packed binary32 operations (each half rounds
// like the scalar operation, in the reference's order). The work is a flat list of tiles of
// kInlierTile candidates over the batch's scans with usable planes (scan by scan, so a tile
// belongs to one scan), taken grid-strided: a large scan spreads over the whole grid instead of
// its own share of it. A CTA's tiles come in increasing order, so it follows the scans with a
// cursor, loads a scan's planes when it reaches it and adds its counts when it leaves it (integer
// partial counts add up exactly).
constexpr uint32_t kInlierTile = 1024;

__global__ void __launch_bounds__(256) k_ransac_inliers(BatchDev b)
{
    static_assert(kMaxRansacIters <= 64, "two planes per lane");
    __shared__ float4 tile[kInlierTile];
    const uint32_t lane = lane_id();
    const uint32_t i0 = lane, i1 = lane + 32u;
    const uint32_t warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    auto tiles_of = [&](int q) -> uint32_t {
        return (b.pvalid[q] != 0ull) ? div_up(b.state[q].n_cand, kInlierTile) : 0u;
    };
    int cs = 0; // the cursor: scan cs owns tiles [cbase, cbase + ctiles)
    uint32_t cbase = 0u, ctiles = (b.nscan > 0) ? tiles_of(0) : 0u;
    int s = -1; // the scan whose planes are loaded
    unsigned long long valid = 0ull;
    float2 qx = make_float2(0.f, 0.f), qy = qx, qz = qx, nqw = qx;
    float thr = 0.0f;
    uint32_t ca = 0u, cb = 0u;
    auto flush = [&]() {
        if (s < 0)
            return;
        if (i0 < static_cast<uint32_t>(kMaxRansacIters) && ((valid >> i0) & 1ull) && ca)
            atomicAdd(&b.inliers[s * kMaxRansacIters + i0], ca);
        if (i1 < static_cast<uint32_t>(kMaxRansacIters) && ((valid >> i1) & 1ull) && cb)
            atomicAdd(&b.inliers[s * kMaxRansacIters + i1], cb);
        ca = cb = 0u;
    };
    for (uint32_t it = blockIdx.x;; it += gridDim.x)
    {
        while (cs < b.nscan && it >= cbase + ctiles)
        {
            cbase += ctiles;
            ++cs;
            ctiles = (cs < b.nscan) ? tiles_of(cs) : 0u;
        }
        if (cs >= b.nscan)
            break; // uniform over the block
        if (cs != s)
        {
            flush();
            s = cs;
            valid = b.pvalid[s];
            const float4 qa = (i0 < static_cast<uint32_t>(kMaxRansacIters)) ? b.planes[s * kMaxRansacIters + i0] : zero;
            const float4 qb = (i1 < static_cast<uint32_t>(kMaxRansacIters)) ? b.planes[s * kMaxRansacIters + i1] : zero;
            qx = make_float2(qa.x, qb.x);
            qy = make_float2(qa.y, qb.y);
            qz = make_float2(qa.z, qb.z);
            nqw = make_float2(-qa.w, -qb.w); // x - w == x + (-w) exactly
            thr = b.scans[s].thr;
        }
        const ScanState& st = b.state[s];
        const uint32_t base = (it - cbase) * kInlierTile;
        const uint32_t cnt = min(kInlierTile, st.n_cand - base);
        const float4* cand = b.cand + st.cand_off + base;
        // candidates staged in shared memory (coalesced), read by each warp as broadcasts
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x)
            tile[k] = cand[k];
        __syncthreads();
#pragma unroll 4
        for (uint32_t k = warp; k < cnt; k += nwarp)
        {
            const float4 p = tile[k];
            float2 t = __fmul2_rn(qx, make_float2(p.x, p.x));
            t = __fadd2_rn(t, __fmul2_rn(qy, make_float2(p.y, p.y)));
            t = __fadd2_rn(t, __fmul2_rn(qz, make_float2(p.z, p.z)));
            t = __fadd2_rn(t, nqw);
            ca += (fabsf(t.x) < thr) ? 1u : 0u;
            cb += (fabsf(t.y) < thr) ? 1u : 0u;
        }
    }
    flush();
}

__global__ void k_ransac_select(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    ScanState& st = b.state[s];
    const unsigned long long valid = b.pvalid[s];
    uint32_t best = 0;
    int bi = -1;
    for (int it = 0; it < kMaxRansacIters; ++it)
    {
        if (!((valid >> it) & 1ull))
            continue;
        const uint32_t c = b.inliers[s * kMaxRansacIters + it];
        if (c > best)
        {
            best = c;
            bi = it;
        }
    }
    if (best > 0)
    {
        float4 q = b.planes[s * kMaxRansacIters + bi];
        if (q.z < 0)
        {
            q.x = -q.x;
            q.y = -q.y;
            q.z = -q.z;
            q.w = -q.w;
        }
        st.plane[0] = q.x;
        st.plane[1] = q.y;
        st.plane[2] = q.z;
        st.plane[3] = q.w;
        st.ransac_ok = 1;
    }
}

// ------------------------------------------------------------------------------------------
// Labels and range-image projection (segmenter.cpp:269-318 + the RANSAC relabel :445-478).
// Per pixel the winner is the lexicographic minimum of (x^2+y^2, cell, cloud index), the
// order in which the reference's strict '<' visits candidates.
// ------------------------------------------------------------------------------------------
__global__ void k_label_depth(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.npts)
        return;
    const int32_t c = b.pt_cell[i];
    const float4 p = b.pts[i];
    const int32_t pix = b.pt_pix[i];
    if (c < 0)
        return;
    const int s = scan_of_point(b, i);
    const ScanDev& sd = b.scans[s];
    const ScanState& st = b.state[s];
    uint8_t lbl = (p.z >= b.elev[c] + sd.thr) ? LP_LABEL_OBSTACLE : LP_LABEL_GROUND;
    const int32_t radial = static_cast<int32_t>((static_cast<uint32_t>(c) - sd.cell_off) % static_cast<uint32_t>(sd.nrad));
    if (radial < kRansacRadialBins && st.ransac_ok)
    {
        const float sdist = (st.plane[0] * p.x) + (st.plane[1] * p.y) + (st.plane[2] * p.z) - st.plane[3];
        if (sdist < sd.thr)
            lbl = LP_LABEL_GROUND;
    }
    b.pt_label[i] = lbl;
    const float d2 = (p.x * p.x) + (p.y * p.y);
    atomicMin(&b.pix_depth[sd.pix_off + static_cast<uint32_t>(pix)], __float_as_uint(d2));
}

__global__ void k_project_key(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.npts)
        return;
    const int32_t c = b.pt_cell[i];
    const float4 p = b.pts[i];
    const int32_t lpix = b.pt_pix[i];
    if (c < 0)
        return;
    const int s = scan_of_point(b, i);
    const ScanDev& sd = b.scans[s];
    const float d2 = (p.x * p.x) + (p.y * p.y);
    const uint32_t pix = sd.pix_off + static_cast<uint32_t>(lpix);
    if (__float_as_uint(d2) != b.pix_depth[pix])
        return;
    const unsigned long long key = (static_cast<unsigned long long>(static_cast<uint32_t>(c) - sd.cell_off) << 32) |
                                   static_cast<unsigned long long>(i - sd.pt_off);
    atomicMin(&b.pix_key[pix], key);
}

__global__ void k_pixel(BatchDev b)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= b.npix)
        return;
    const unsigned long long key = b.pix_key[p];
    if (key == ~0ull)
    {
        b.pix_map[p] = -1;
        b.pix_state[p] = PX_EMPTY;
        return;
    }
    const int s = scan_of_pix(b, p);
    const uint32_t li = static_cast<uint32_t>(key & 0xffffffffull);
    b.pix_map[p] = static_cast<int32_t>(li);
    b.pix_state[p] = (b.pt_label[b.scans[s].pt_off + li] == LP_LABEL_GROUND) ? PX_GROUND : PX_OBSTACLE;
}

// ------------------------------------------------------------------------------------------
// Dilation of the obstacle channel by a 5x5 rectangle clipped at the image border, and the
// row-major intersection queue (segmenter.cpp:486-514): one block per image row.
// ------------------------------------------------------------------------------------------
// Bit-mask form: a warp takes 32 consecutive pixels at a time; a ballot over each of the five
// rows h-2..h+2 gives the obstacle bits of that segment, the rows are OR-ed, and the +-2 column
// dilation is done with shifts, the two halo bits on each side coming from the neighbouring
// segments (zero outside the image: the rectangle is clipped at the border). Dilation changes
// only ground and empty pixels, never the obstacle channel, so rows are independent. Each warp
// walks a contiguous run of segments; the queue keeps column order through per-warp counts.
__device__ __forceinline__ uint32_t obstacle_bits(const uint8_t* st, int32_t H, int32_t W, int32_t h, int32_t seg)
{
    uint32_t m = 0u;
    const int32_t w = seg * 32 + static_cast<int32_t>(lane_id());
    const bool colok = seg >= 0 && w < W;
#pragma unroll
    for (int32_t dh = -2; dh <= 2; ++dh)
    {
        const int32_t hh = h + dh;
        const bool ok = colok && hh >= 0 && hh < H;
        m |= __ballot_sync(0xffffffffu, ok && st[hh * W + w] == PX_OBSTACLE);
    }
    return m;
}

__global__ void __launch_bounds__(256) k_dilate_rows(BatchDev b)
{
    __shared__ uint32_t wcount[8];
    __shared__ uint32_t woff[8];
    const uint32_t r = blockIdx.x;
    const int s = scan_of_row(b, r);
    const ScanDev& sd = b.scans[s];
    const int32_t h = static_cast<int32_t>(r - sd.row_off);
    const int32_t H = sd.H, W = sd.W;
    uint8_t* st = b.pix_state + sd.pix_off;
    const uint32_t row_base = sd.pix_off + static_cast<uint32_t>(h * W);
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    const int32_t nseg = (W + 31) / 32;
    const int32_t per = (nseg + 7) / 8;
    const int32_t s0 = static_cast<int32_t>(warp) * per, s1 = min(nseg, s0 + per);
    // pass 1: dilate, update the states, count the queued (ground -> intersection) pixels
    uint32_t count = 0u;
    uint32_t left = (s0 < s1) ? obstacle_bits(st, H, W, h, s0 - 1) : 0u;
    uint32_t cur = (s0 < s1) ? obstacle_bits(st, H, W, h, s0) : 0u;
    for (int32_t seg = s0; seg < s1; ++seg)
    {
        const uint32_t right = obstacle_bits(st, H, W, h, seg + 1);
        const uint32_t d = cur | (cur << 1) | (cur << 2) | (cur >> 1) | (cur >> 2) | (left >> 31) | (left >> 30) |
                           (right << 31) | (right << 30);
        const int32_t w = seg * 32 + static_cast<int32_t>(lane);
        bool inter = false;
        if (w < W && ((d >> lane) & 1u))
        {
            const uint8_t c = st[h * W + w];
            if (c == PX_GROUND)
            {
                inter = true;
                st[h * W + w] = PX_INTERSECT;
            }
            else if (c == PX_EMPTY)
                st[h * W + w] = PX_EMPTY_RED;
        }
        count += static_cast<uint32_t>(__popc(__ballot_sync(0xffffffffu, inter)));
        left = cur;
        cur = right;
    }
    if (lane == 0)
        wcount[warp] = count;
    __syncthreads();
    __shared__ uint32_t qbase;
    if (threadIdx.x == 0)
    {
        uint32_t run = 0u;
        for (int k = 0; k < 8; ++k)
        {
            woff[k] = run;
            run += wcount[k];
        }
        b.row_cnt[r] = run;
        // the row's segment of the flat list of queued pixels (row_cnt[nrows] counts them); the
        // capacity bound (a queued pixel holds a point) cannot be exceeded, checked all the same
        qbase = run ? atomicAdd(&b.row_cnt[b.nrows], run) : 0u;
        if (qbase + run > b.jq_cap)
        {
            raise_err(&b.state[s], ERR_INTERNAL);
            b.row_cnt[r] = 0u;
            qbase = 0u;
        }
        b.row_q0[r] = qbase;
    }
    __syncthreads();
    // pass 2: queue entries in column order (this row's states now hold the intersections)
    uint32_t pos = woff[warp];
    for (int32_t seg = s0; seg < s1; ++seg)
    {
        const int32_t w = seg * 32 + static_cast<int32_t>(lane);
        const bool inter = w < W && st[h * W + w] == PX_INTERSECT;
        const uint32_t m = __ballot_sync(0xffffffffu, inter);
        if (inter)
        {
            const uint32_t j = pos + static_cast<uint32_t>(__popc(m & ((1u << lane) - 1u)));
            b.row_cols[row_base + j] = static_cast<uint16_t>(w);
            // (row, position | column << 16, the pixel's point, scan): the weights pass starts here
            if (qbase + j < b.jq_cap)
                b.jq[qbase + j] = make_uint4(r, j | (static_cast<uint32_t>(w) << 16),
                                         static_cast<uint32_t>(b.pix_map[sd.pix_off + static_cast<uint32_t>(h * W + w)]),
                                         static_cast<uint32_t>(s));
        }
        pos += static_cast<uint32_t>(__popc(m));
    }
}

// Offsets of the 24-neighbour kernel (segmenter.cpp:527-530: the 5x5 window without its centre,
// row-major) as arithmetic on the slot index (folds to constants in unrolled loops).
__device__ __forceinline__ constexpr int32_t jcp_dh(int k)
{
    return k < 10 ? -2 + k / 5 : (k < 14 ? 0 : 1 + (k - 14) / 5);
}
__device__ __forceinline__ constexpr int32_t jcp_dw(int k)
{
    return k < 10 ? k % 5 - 2 : (k < 14 ? (k < 12 ? k - 12 : k - 11) : (k - 14) % 5 - 2);
}

__device__ __forceinline__ uint8_t final_view(uint8_t st)
{
    return (st == PX_GROUND || st == PX_RES_G) ? V_G : ((st == PX_OBSTACLE || st == PX_RES_O) ? V_O : V_U);
}
__device__ __forceinline__ uint8_t pre_view(uint8_t st)
{
    return (st == PX_GROUND) ? V_G : ((st == PX_OBSTACLE) ? V_O : V_U);
}

// A queued pixel's vote (segmenter.cpp:585-631) as a 9-state transition map of the in-row chain.
// The reference sums, in slot order, the normalised weights of the slots labelled ground into g
// and of those labelled obstacle into o (a slot with another label adds nothing), and votes
// obstacle iff o > g. Here both sums run as one pair (a slot adds (w, 0), (0, w) or (0, 0);
// weights and sums are never negative, so adding +0 is exactly the reference's skip, and each half
// rounds like its scalar addition in the same order). The labels at slots 10 (column c-2) and 11
// (c-1) are symbolic where those are queued pixels of the same row (their outcomes, the chain's
// state; sym_b / sym_a). g after slot 11 is one of four values (whether slot 10, then slot 11, is
// ground) and so is o, so four chains over slots 12-23 give the final sums for all nine label
// pairs of slots 10 and 11 (an outcome table of 2 bits per pair); each chain state reads the
// pair its labels select. The map (state = 3 x + a) is built for the column gap to the previous
// queued pixel.
__device__ __forceinline__ unsigned long long vote_map(const float* wn, const uint8_t* lb, bool sym_a, bool sym_b,
                                                       bool live, int32_t gap)
{
    auto gw = [](uint8_t l, float w) { return make_float2(l == V_G ? w : 0.0F, l == V_O ? w : 0.0F); };
    float2 head = make_float2(0.0F, 0.0F);
#pragma unroll
    for (int k = 0; k < 10; ++k)
        head = __fadd2_rn(head, gw(lb[k], wn[k]));
    // start i (bit 0: slot 10 adds, bit 1: slot 11 adds): g in .x, o in .y, each slot added in order
    float2 v[4];
    v[0] = head;
    v[1] = __fadd2_rn(head, make_float2(wn[10], wn[10]));
    v[2] = __fadd2_rn(head, make_float2(wn[11], wn[11]));
    v[3] = __fadd2_rn(v[1], make_float2(wn[11], wn[11]));
#pragma unroll
    for (int k = 12; k < 24; ++k)
    {
        const float2 d = gw(lb[k], wn[k]);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            v[i] = __fadd2_rn(v[i], d);
    }
    // outcome of label pair (l10, l11) at bits 2 (3 l10 + l11): the starts it selects are fixed
    uint32_t otab = 0u;
#pragma unroll
    for (int l10 = 0; l10 < 3; ++l10)
#pragma unroll
        for (int l11 = 0; l11 < 3; ++l11)
        {
            const int ig = (l10 == V_G ? 1 : 0) | (l11 == V_G ? 2 : 0);
            const int io = (l10 == V_O ? 1 : 0) | (l11 == V_O ? 2 : 0);
            otab |= static_cast<uint32_t>((v[io].y > v[ig].x) ? V_O : V_G) << (2 * (3 * l10 + l11));
        }
    if (!live)
        otab = 0u; // V_U whatever the labels
    const int g1 = gap == 1, g2 = gap == 2;
    unsigned long long t = 0ull;
#pragma unroll
    for (int sidx = 0; sidx < 9; ++sidx)
    {
        const int a = sidx / 3, bb = sidx % 3;
        const int ap = g1 ? a : V_U;
        const int bp = g1 ? bb : (g2 ? a : V_U);
        const int l10 = sym_b ? bp : lb[10];
        const int l11 = sym_a ? ap : lb[11];
        const uint32_t x = (otab >> (2 * (3 * l10 + l11))) & 3u;
        t |= static_cast<unsigned long long>(3u * x + static_cast<uint32_t>(ap)) << (4 * sidx);
    }
    return t;
}

// Fresh (not stale) weight of every in-bounds neighbour slot of every queued pixel: 0 for an
// empty neighbour or one farther than the kernel threshold, else expf(-amp * dist)
// (segmenter.cpp:545-607). These depend on geometry only, so they are computed in parallel
// before the ordered vote. Two records per queued pixel:
//   jw: the raw weights and their sum (read back when a later pixel's slot leaves the image;
//       written for the last three queued pixels of each row, the only ones read),
//   jn: the weights divided by the sum, the sum, and a 2-bit label code per slot: the label the
//       vote will read (unknown / ground / obstacle) wherever it is already fixed, or 3 where it
//       is not: a queued pixel in a row above (its final colour comes from its own vote) or a
//       queued pixel to the left in the same row (the symbolic outcome of the in-row chain).
__global__ void __launch_bounds__(256) k_jcp_weights(BatchDev b)
{
    // one warp per queued pixel of the batch's flat list (rows of any length spread over the whole
    // grid), lane k = kernel slot k (lanes 24-31 idle); the weights are summed by lane 0 in slot
    // order, as the reference's loop adds them
    const uint32_t total = min(b.row_cnt[b.nrows], b.jq_cap);
    const uint32_t lane = lane_id();
    const int k = static_cast<int>(lane);
    const int32_t dh = jcp_dh(k), dw = jcp_dw(k);
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < total; q += nw)
    {
        const uint4 e = b.jq[q];
        const uint32_t r = e.x, j = e.y & 0xffffu;
        const int32_t w = static_cast<int32_t>(e.y >> 16);
        const int s = static_cast<int>(e.w);
        const ScanDev& sd = b.scans[s];
        const int32_t h = static_cast<int32_t>(r - sd.row_off);
        const int32_t H = sd.H, W = sd.W;
        const uint32_t row_base = sd.pix_off + static_cast<uint32_t>(h * W);
        const uint32_t m = b.row_cnt[r];
        const int32_t* map = b.pix_map + sd.pix_off;
        const uint8_t* st = b.pix_state + sd.pix_off;
        const float4* pts = b.pts + sd.pt_off;
        const float4 cp = pts[e.z];
        float wt = 0.0F;
        uint32_t code = V_U;
        const int32_t hh = h + dh, ww = w + dw;
        if (k < 24 && hh >= 0 && hh < H && ww >= 0 && ww < W)
        {
            const int32_t ni = map[hh * W + ww];
            if (ni >= 0)
            {
                const float4 np = pts[ni];
                const float dx = cp.x - np.x;
                const float dy = cp.y - np.y;
                const float dz = cp.z - np.z;
                const float d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 > sd.kthr2))
                    wt = lpm::cr_expf(-sd.amp * sqrtf(d2));
            }
            if (wt != 0.0F)
            {
                const uint8_t ns = st[hh * W + ww];
                if (dh > 0 || (dh == 0 && dw > 0))
                    code = pre_view(ns); // not voted before this pixel
                else
                    code = (ns == PX_INTERSECT) ? 3u : final_view(ns);
            }
        }
        float sum = 0.0F;
#pragma unroll
        for (int q = 0; q < 24; ++q)
            sum += __shfl_sync(0xffffffffu, wt, q);
        unsigned long long codes = (k < 24) ? (static_cast<unsigned long long>(code) << (2 * k)) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            codes |= __shfl_xor_sync(0xffffffffu, codes, o);
        const bool live = fabsf(sum) > FLT_EPSILON;
        // the raw record is only read for the row's last three queued pixels (the stale-slot
        // sources of later rows and of the row's right border)
        const bool raw = j + 3u >= m;
        // raw records: the row's last three positions, slot j + 3 - m; normalised: by queue position
        float* out = raw ? b.jw + (static_cast<size_t>(r) * 3u + (j + 3u - m)) * kJwStride : nullptr;
        float* nrm = b.jn + static_cast<size_t>(q) * kJwStride;
        if (k < 24)
        {
            if (raw)
                out[k] = wt;
            nrm[k] = live ? wt / sum : 0.0F;
        }
        else if (k < 28)
        {
            if (raw)
                out[k] = (k == 24) ? sum : 0.0F;
            nrm[k] = (k == 24) ? sum
                               : ((k == 25) ? __uint_as_float(static_cast<uint32_t>(codes))
                                            : ((k == 26) ? __uint_as_float(static_cast<uint32_t>(codes >> 32)) : 0.0F));
        }
    }
}

// Row record of the ordered vote (kJrowWords words per image row with queued pixels), one warp per
// row (lanes 0-23: slots), after k_jcp_weights has written every pixel's raw weight record.
__global__ void __launch_bounds__(256) k_jcp_rowrec(BatchDev b)
{
    const uint32_t r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (r >= b.nrows || lane_id() >= 24u)
        return;
    const uint32_t m = b.row_cnt[r];
    if (m == 0u)
        return;
    const int s = scan_of_row(b, r);
    const ScanDev& sd = b.scans[s];
    const int32_t h = static_cast<int32_t>(r - sd.row_off);
    const int32_t H = sd.H, W = sd.W;
    const uint32_t row_base = sd.pix_off + static_cast<uint32_t>(h * W);
    const uint8_t* st = b.pix_state + sd.pix_off;

    // Row record (kJrowWords words): lastq[d] = the last of the row's final three queued pixels
    // with column <= W-1-d; per slot k, what the row leaves in the reference's stale weight/label
    // buffer: the raw weight of the last queued pixel for which slot k is inside the image, and
    // its label, fixed already or (a queued pixel before it in vote order) read after the vote.
    uint32_t* rec = b.jrow + static_cast<size_t>(r) * kJrowWords;
    const uint16_t* cols = b.row_cols + row_base;
    int32_t lq[3];
    for (int32_t d = 0; d < 3; ++d)
    {
        lq[d] = -1;
        for (int32_t j = static_cast<int32_t>(m) - 1; j >= 0 && j >= static_cast<int32_t>(m) - 3; --j)
            if (cols[j] <= W - 1 - d)
            {
                lq[d] = j;
                break;
            }
    }
    const int k = static_cast<int>(lane_id());
    if (k < 3)
        rec[k] = static_cast<uint32_t>(lq[k]);
    const int32_t dh = jcp_dh(k), dw = jcp_dw(k);
    const int32_t hh = h + dh;
    uint32_t info = kJrowNoUpdate;
    float qw = 0.0F;
    if (hh >= 0 && hh < H)
    {
        const int32_t q = lq[dw > 0 ? dw : 0];
        if (q >= 0 && static_cast<int32_t>(cols[q]) >= (dw < 0 ? -dw : 0))
        {
            qw = b.jw[(static_cast<size_t>(r) * 3u + static_cast<uint32_t>(q + 3 - static_cast<int32_t>(m))) * kJwStride + k];
            info = V_U;
            if (qw != 0.0F)
            {
                const uint32_t addr = static_cast<uint32_t>(hh * W + cols[q] + dw);
                const uint8_t ns = st[addr];
                const bool before = (dh < 0) || (dh == 0 && dw < 0);
                if (!before)
                    info = pre_view(ns);
                else if (ns == PX_INTERSECT)
                    info = kJrowDynamic | addr; // its colour is its own vote's outcome
                else
                    info = final_view(ns);
            }
        }
    }
    rec[4 + k] = __float_as_uint(qw);
    rec[28 + k] = info;
}

__device__ __forceinline__ unsigned long long map_compose(unsigned long long later, unsigned long long earlier)
{
    unsigned long long r = 0ull;
#pragma unroll
    for (int s = 0; s < 9; ++s)
    {
        const uint32_t mid = static_cast<uint32_t>((earlier >> (4 * s)) & 0xfull);
        r |= ((later >> (4 * mid)) & 0xfull) << (4 * s);
    }
    return r;
}
__device__ __forceinline__ unsigned long long map_identity()
{
    unsigned long long r = 0ull;
#pragma unroll
    for (int s = 0; s < 9; ++s)
        r |= static_cast<unsigned long long>(s) << (4 * s);
    return r;
}

// The ordered vote (segmenter.cpp:535-637), one block per scan, image rows in order.
//
// Within a row, the queued pixel at column c reads the vote outcomes of the queued pixels at
// c-1 and c-2 (already written in the reference's FIFO); everything else it reads is fixed:
// rows above are final, rows below and columns to the right still hold their pre-vote colour.
// Each queued pixel therefore has a vote table f(a, b) over the outcomes a (column c-1) and
// b (column c-2), each in {unknown, ground, obstacle}; the row is a chain of 9-state
// transitions composed by a block-wide prefix scan, which reproduces the FIFO exactly.
//
// Slots outside the image keep the weight and label the previous queued pixel wrote to that
// slot (segmenter.cpp:552-556). That pixel is the last earlier queued pixel for which the slot
// was inside the image: for a right-border pixel it can be an earlier pixel of the same row
// (columns <= W-1-dw); otherwise it lies in an earlier row, tracked as a running value per
// slot across rows.
__global__ void __launch_bounds__(256) k_jcp_rows(BatchDev b)
{
    __shared__ float run_w[24];
    __shared__ uint8_t run_l[24];
    __shared__ unsigned long long wmaps[8];
    __shared__ unsigned long long rmap[256]; // a row's maps by position (rows of at most 256 pixels)
    // final colour (V_U/V_G/V_O) of the queued pixels of the last three rows, by column: the
    // labels a pixel reads from queued pixels above it, without a global load (images up to
    // kFinRingW columns; wider ones read the pixel states)
    __shared__ uint8_t fin[3][kFinRingW];
    // Double-buffered staging: while a row votes, one thread copies the next non-empty row's
    // normalised records and queue entries into shared memory with a TMA bulk copy (rows of at
    // most kStageRec queued pixels, images of at most kRowCache rows; others load directly).
    extern __shared__ __align__(16) unsigned char stage[];
    __shared__ uint32_t mrow[kRowCache];
    __shared__ unsigned long long mbar[2];
    __shared__ int32_t st_row[2], st_coff[2];
    __shared__ int32_t st_pend[2]; // a copy into the buffer is in flight (issued, not yet waited for)
    const int s = blockIdx.x;
    const ScanDev& sd = b.scans[s];
    const int32_t H = sd.H, W = sd.W;
    const bool ring = W <= static_cast<int32_t>(kFinRingW);
    const bool cache = H <= static_cast<int32_t>(kRowCache);
    if (cache)
        for (int32_t i = threadIdx.x; i < H; i += blockDim.x)
            mrow[i] = b.row_cnt[sd.row_off + static_cast<uint32_t>(i)];
    if (threadIdx.x == 0)
    {
        mbar_init(&mbar[0], 1u);
        mbar_init(&mbar[1], 1u);
        st_row[0] = st_row[1] = -1;
        st_pend[0] = st_pend[1] = 0;
    }
    __syncthreads();
    // thread 0: copy row hh into buffer bf (queue entries widened to 16-byte bounds)
    auto issue = [&](int32_t hh, int bf) {
        const uint32_t mm = mrow[hh];
        const uint32_t rb = sd.pix_off + static_cast<uint32_t>(hh * W);
        const uint32_t rec_bytes = mm * kJwStride * 4u;
        const uintptr_t c0 = reinterpret_cast<uintptr_t>(b.row_cols + rb);
        const uintptr_t ca = c0 & ~static_cast<uintptr_t>(15);
        const uintptr_t ce = (reinterpret_cast<uintptr_t>(b.row_cols + rb + mm) + 15) & ~static_cast<uintptr_t>(15);
        unsigned char* dst = stage + bf * kStageBytes;
        mbar_expect_tx(&mbar[bf], rec_bytes + static_cast<uint32_t>(ce - ca) + kJrowWords * 4u);
        bulk_g2s(dst, b.jn + static_cast<size_t>(b.row_q0[sd.row_off + static_cast<uint32_t>(hh)]) * kJwStride, rec_bytes,
                 &mbar[bf]);
        bulk_g2s(dst + kStageRecBytes, reinterpret_cast<const void*>(ca), static_cast<uint32_t>(ce - ca), &mbar[bf]);
        bulk_g2s(dst + kStageRecBytes + kStageColBytes,
                 b.jrow + static_cast<size_t>(sd.row_off + static_cast<uint32_t>(hh)) * kJrowWords, kJrowWords * 4u,
                 &mbar[bf]);
        st_row[bf] = hh;
        st_coff[bf] = static_cast<int32_t>((c0 - ca) / 2);
        st_pend[bf] = 1;
    };
    auto stageable = [&](int32_t hh) { return cache && mrow[hh] > 0 && mrow[hh] <= kStageRec; };
    auto next_row = [&](int32_t hh) {
        for (int32_t q = hh + 1; q < H; ++q)
            if (mrow[q] > 0)
                return q;
        return -1;
    };
    uint32_t parity[2] = {0u, 0u};
    int cur = 0;
    if (threadIdx.x == 0 && cache)
    {
        const int32_t h0 = next_row(-1);
        if (h0 >= 0 && stageable(h0))
            issue(h0, 0);
    }
    __syncthreads();
    uint8_t* st = b.pix_state + sd.pix_off;
    if (threadIdx.x < 24)
    {
        run_w[threadIdx.x] = 0.0F;
        run_l[threadIdx.x] = V_U;
    }
    __syncthreads();
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5;
    for (int32_t h = 0; h < H; ++h)
    {
        const uint32_t r = sd.row_off + static_cast<uint32_t>(h);
        const uint32_t m = cache ? mrow[h] : b.row_cnt[r];
        if (m == 0)
            continue;
        const uint32_t row_base = sd.pix_off + static_cast<uint32_t>(h * W);
        const uint16_t* cols = b.row_cols + row_base;
        const uint32_t q0 = b.row_q0[r]; // the row's first position in the flat queue
        const bool staged = st_row[cur] == h;
        const float4* srec = reinterpret_cast<const float4*>(stage + cur * kStageBytes);
        const uint16_t* scols = reinterpret_cast<const uint16_t*>(stage + cur * kStageBytes + kStageRecBytes) + st_coff[cur];
        __syncthreads(); // every thread has read st_row / st_coff before thread 0 reissues
        if (threadIdx.x == 0 && cache)
        {
            const int32_t hn = next_row(h);
            st_row[cur ^ 1] = -1;
            if (hn >= 0 && stageable(hn))
                issue(hn, cur ^ 1);
        }
        if (staged)
        {
            // every thread waits (bounded); the block decides together whether the copy landed
            const bool landed = mbar_wait(&mbar[cur], parity[cur], 1u << 22);
            if (!__syncthreads_and(landed))
            {
                // report, then give every copy still in flight (this row's and the next row's,
                // issued above) a last bounded wait before the CTA leaves its shared memory
                if (threadIdx.x == 0)
                    raise_err(&b.state[s], ERR_INTERNAL);
                for (int bf = 0; bf < 2; ++bf)
                    if (st_pend[bf])
                        mbar_wait(&mbar[bf], parity[bf], 1u << 24);
                return;
            }
            parity[cur] ^= 1u;
            // landed for every thread, so no thread reads st_pend in this row; thread 0 alone
            // writes it (here and in issue), so clearing needs no further barrier
            if (threadIdx.x == 0)
                st_pend[cur] = 0;
        }
        // the row's record (from the parallel pass): lastq and the stale-buffer update
        const uint32_t* rrec = staged ? reinterpret_cast<const uint32_t*>(stage + cur * kStageBytes + kStageRecBytes + kStageColBytes)
                                      : b.jrow + static_cast<size_t>(r) * kJrowWords;
        const int32_t lastq[3] = {static_cast<int32_t>(rrec[0]), static_cast<int32_t>(rrec[1]),
                                  static_cast<int32_t>(rrec[2])};
        float upd_w = 0.0F;
        uint32_t upd_info = kJrowNoUpdate;
        if (threadIdx.x < 24)
        {
            upd_w = __uint_as_float(rrec[4 + threadIdx.x]);
            upd_info = rrec[28 + threadIdx.x];
        }

        // ---- per queued pixel: vote table -> 9-state transition map --------------------------
        const int32_t fr2 = (h + 1) % 3, fr1 = (h + 2) % 3; // final-colour rows of h-2 and h-1
        // Consecutive chunks of pixels per thread (one pixel per thread in rows of at most 256
        // pixels, whose maps stay in shared memory).
        const bool spread = m <= blockDim.x;
        const uint32_t chunk = (m + blockDim.x - 1) / blockDim.x;
        const uint32_t j0 = threadIdx.x * chunk;
        const uint32_t j1 = min(m, j0 + chunk);
        unsigned long long agg = map_identity();
        for (uint32_t j = j0; j < j1; ++j)
        {
            // the pixel's queue entry and normalised record: staged in shared memory, or loaded
            const int32_t c = staged ? scols[j] : cols[j];
            const float4* rec = staged ? srec + 7u * j
                                       : reinterpret_cast<const float4*>(b.jn + static_cast<size_t>(q0 + j) * kJwStride);
            float wn[24];
#pragma unroll
            for (int q = 0; q < 6; ++q)
            {
                const float4 v = rec[q];
                wn[4 * q] = v.x;
                wn[4 * q + 1] = v.y;
                wn[4 * q + 2] = v.z;
                wn[4 * q + 3] = v.w;
            }
            const float4 tail = rec[6];
            const float sum = tail.x;
            const unsigned long long codes =
                static_cast<unsigned long long>(__float_as_uint(tail.y)) |
                (static_cast<unsigned long long>(__float_as_uint(tail.z)) << 32);
            unsigned long long t;
            if (h >= 2 && h + 2 < H && c >= 2 && c + 2 < W)
            {
                // the window lies inside the image: labels from the codes and the final colours
                // above (no stale slot)
                const bool live = fabsf(sum) > FLT_EPSILON;
                uint8_t lb[24];
                bool sym_a = false, sym_b = false;
#pragma unroll
                for (int k = 0; k < 24; ++k)
                {
                    const uint32_t code = static_cast<uint32_t>((codes >> (2 * k)) & 3ull);
                    if (code != 3u)
                        lb[k] = static_cast<uint8_t>(code);
                    else if (k < 10)
                    {
                        const int32_t hh = h + jcp_dh(k), ww = c + jcp_dw(k);
                        lb[k] = ring ? fin[k < 5 ? fr2 : fr1][ww] : final_view(st[hh * W + ww]);
                    }
                    else
                    {
                        lb[k] = V_U; // same row, left of c, queued: the chain's state
                        if (k == 11)
                            sym_a = true;
                        else
                            sym_b = true;
                    }
                }
                const int32_t gap = (j > 0) ? (c - static_cast<int32_t>(staged ? scols[j - 1] : cols[j - 1])) : 1000;
                t = vote_map(wn, lb, sym_a, sym_b, live, gap);
            }
            else
            {
                uint8_t nsv[10]; // final colour of the queued pixels above (code 3: inside the image)
#pragma unroll
                for (int k = 0; k < 10; ++k)
                {
                    const int32_t hh = h + jcp_dh(k), ww = c + jcp_dw(k);
                    nsv[k] = V_U;
                    if (((codes >> (2 * k)) & 3ull) == 3ull)
                        nsv[k] = ring ? fin[hh % 3][ww] : final_view(st[hh * W + ww]);
                }
                const bool live = fabsf(sum) > FLT_EPSILON;
                uint8_t lb[24];
                bool sym_a = false, sym_b = false;
#pragma unroll
                for (int k = 0; k < 24; ++k)
                {
                    const int32_t dh = jcp_dh(k), dw = jcp_dw(k);
                    const int32_t hh = h + dh, ww = c + dw;
                    if (hh < 0 || hh >= H || ww < 0 || ww >= W)
                    {
                        // stale slot: the raw weight an earlier pixel left there, over this sum
                        float wv = 0.0F;
                        lb[k] = V_U;
                        if (live)
                        {
                            const int32_t qd = dw > 0 ? dw : 0;
                            const int32_t q = (dw > 0 && hh >= 0 && hh < H) ? lastq[qd] : -1;
                            if (q >= 0)
                            {
                                const float qw = b.jw[(static_cast<size_t>(r) * 3u + static_cast<uint32_t>(q + 3 - static_cast<int32_t>(m))) * kJwStride + k];
                                wv = qw;
                                if (qw != 0.0F)
                                {
                                    const uint8_t ns = st[hh * W + cols[q] + dw];
                                    lb[k] = (dh < 0) ? final_view(ns) : pre_view(ns);
                                }
                            }
                            else
                            {
                                wv = run_w[k];
                                lb[k] = run_l[k];
                            }
                            wn[k] = wv / sum;
                        }
                        continue;
                    }
                    const uint32_t code = static_cast<uint32_t>((codes >> (2 * k)) & 3ull);
                    if (code != 3u)
                        lb[k] = static_cast<uint8_t>(code);
                    else if (dh < 0)
                        lb[k] = nsv[k < 10 ? k : 0];
                    else
                    {
                        // same row, left of c, queued: symbolic (the chain's outcome)
                        lb[k] = V_U;
                        if (dw == -1)
                            sym_a = true;
                        else
                            sym_b = true;
                    }
                }
                const int32_t gap = (j > 0) ? (c - static_cast<int32_t>(staged ? scols[j - 1] : cols[j - 1])) : 1000;
                t = vote_map(wn, lb, sym_a, sym_b, live, gap);
            }
            if (spread)
                rmap[j] = t;
            else
                b.jmap[q0 + j] = t;
            agg = (j == j0) ? t : map_compose(t, agg);
        }

        // ---- block-wide exclusive scan of the thread aggregates (composition order) -----------
        // only the warps holding pixels scan (the others' aggregates are the identity)
        const uint32_t wused = ((m + chunk - 1) / chunk + 31u) / 32u;
        unsigned long long incl = agg;
        if (warp < wused)
        {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const unsigned long long other = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= static_cast<uint32_t>(o))
                    incl = map_compose(incl, other);
            }
        }
        if (lane == 31)
            wmaps[warp] = incl;
        __syncthreads();
        unsigned long long wpre = map_identity();
        for (uint32_t w2 = 0; w2 < min(warp, wused); ++w2)
            wpre = map_compose(wmaps[w2], wpre);
        unsigned long long excl = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0)
            excl = map_identity();
        excl = map_compose(excl, wpre);
        // state before this thread's chunk, starting from (unknown, unknown)
        uint32_t state = static_cast<uint32_t>(excl & 0xfull);
        for (uint32_t j = j0; j < j1; ++j)
        {
            state = static_cast<uint32_t>(((spread ? rmap[j] : b.jmap[q0 + j]) >> (4 * state)) & 0xfull);
            const uint32_t x = state / 3;
            if (x != V_U)
                st[h * W + cols[j]] = (x == V_O) ? PX_RES_O : PX_RES_G;
            if (ring)
                fin[h % 3][cols[j]] = static_cast<uint8_t>(x); // final_view of the new state
        }
        __syncthreads();

        // ---- running stale values: last queued pixel of this row with the slot in bounds ------
        if (upd_info != kJrowNoUpdate)
        {
            run_w[threadIdx.x] = upd_w;
            uint8_t l = static_cast<uint8_t>(upd_info);
            if (upd_info & kJrowDynamic)
            {
                const uint32_t addr = upd_info & ~kJrowDynamic; // a queued pixel of rows h-2..h
                l = ring ? fin[(addr / static_cast<uint32_t>(W)) % 3u][addr % static_cast<uint32_t>(W)]
                         : final_view(st[addr]);
            }
            run_l[threadIdx.x] = l;
        }
        // no barrier here: the next row's first barrier orders these writes before its readers
        cur ^= 1;
    }
}

// populateLabels (segmenter.cpp:640-669) and the colour image of Segmenter::image().
__global__ void k_populate(BatchDev b, uint8_t* image)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= b.npix)
        return;
    const uint8_t stv = b.pix_state[p];
    const int32_t li = b.pix_map[p];
    if (li >= 0)
    {
        const int s = scan_of_pix(b, p);
        const uint8_t v = final_view(stv);
        if (v != V_U)
            b.seg_label[b.scans[s].pt_off + static_cast<uint32_t>(li)] = (v == V_G) ? LP_LABEL_GROUND : LP_LABEL_OBSTACLE;
    }
    if (image)
    {
        uint8_t bgr[3] = {0, 0, 0};
        switch (stv)
        {
        case PX_GROUND:
        case PX_RES_G:
            bgr[1] = 255;
            break;
        case PX_OBSTACLE:
        case PX_RES_O:
        case PX_EMPTY_RED:
            bgr[2] = 255;
            break;
        case PX_INTERSECT:
            bgr[0] = 255;
            break;
        default:
            break;
        }
        image[3 * p] = bgr[0];
        image[3 * p + 1] = bgr[1];
        image[3 * p + 2] = bgr[2];
    }
}
} // namespace

// ------------------------------------------------------------------------------------------
// Host launch sequence for the segmentation stage (all launches on one stream, no host sync).
// ------------------------------------------------------------------------------------------
void launch_ring_only(Launcher& L, const BatchDev& b, const BatchHost& hb)
{
    const uint32_t T = 256;
    LP_LAUNCH(L, k_quadrant, div_up(b.npts, T), T, b);
    LP_LAUNCH(L, k_ring_count, hb.ntiles, 256, b);
    L.scan(b.tile_cnt, b.tile_cnt, hb.ntiles + 1);
    LP_LAUNCH(L, k_ring_apply, hb.ntiles, 256, b);
}

__global__ void k_debug_math(int kind, const float* a, const float* bb, uint32_t n, float* out)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float r;
    switch (kind)
    {
    case 0:
        r = lpm::cr_atan2f(a[i], bb[i]);
        break;
    case 1:
        r = lpm::cr_atanf(a[i]);
        break;
    case 2:
        r = lpm::cr_expf(a[i]);
        break;
    case 4:
        r = lpm::cr_atan2f_fp64(a[i], bb[i]);
        break;
    case 5:
        r = lpm::cr_atanf_fp64(a[i]);
        break;
    case 6:
        r = lpm::cr_expf_fp64(a[i]);
        break;
    default:
        r = lpm::atan2_approx(a[i], bb[i]);
        break;
    }
    out[i] = r;
}

void init_segment_tables()
{
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (dev >= 0 && dev < 64 && done[dev])
        return;
    std::mt19937 gen(42u);
    uint32_t table[kMtTable];
    for (int k = 0; k < kMtTable; ++k)
        table[k] = static_cast<uint32_t>(gen());
    const bool attr = cudaFuncSetAttribute(k_jcp_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(2u * kStageBytes)) == cudaSuccess;
    if (cudaMemcpyToSymbol(g_mt42, table, sizeof(table)) == cudaSuccess && attr && dev >= 0 && dev < 64)
        done[dev] = true;
}

void launch_debug_math(Launcher& L, int kind, const float* a, const float* bb, uint32_t n, float* out)
{
    LP_LAUNCH(L, k_debug_math, div_up(n, 256u), 256, kind, a, bb, n, out);
}

__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Sweep of the float-float first stage against the binary64 / double-double stages. kind 1
// (atan) and 2 (exp): argument = the float whose bits are `first + i`; kind 0 (atan2): (y, x) from
// a hash of first + i, either arbitrary finite floats or the same with their exponents drawn
// close (ratios near 1, the axes and the diagonals). stats: [0] decided by stage 1, [1] left to
// the later stages, [2] stage 1 decided differently; first_bad: lowest such index.
__global__ void k_debug_math_sweep(int kind, unsigned long long first, unsigned long long count,
                                   unsigned long long* stats, unsigned long long* first_bad)
{
    unsigned long long dec = 0, und = 0, bad = 0;
    const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * blockDim.x;
    for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < count;
         i += stride)
    {
        const unsigned long long idx = first + i;
        float f = 0.0f, want = 0.0f;
        bool ok = false;
        if (kind == 1)
        {
            const float x = __uint_as_float(static_cast<uint32_t>(idx));
            ok = lpm::ff_atanf(x, &f);
            if (ok)
                want = lpm::cr_atanf_fp64(x);
        }
        else if (kind == 2)
        {
            const float x = __uint_as_float(static_cast<uint32_t>(idx));
            ok = x >= -87.0f && x <= 88.5f && lpm::ff_expf(x, &f);
            if (ok)
                want = lpm::cr_expf_fp64(x);
        }
        else
        {
            const unsigned long long h = splitmix64(idx);
            uint32_t by = static_cast<uint32_t>(h), bx = static_cast<uint32_t>(h >> 32);
            if (idx & 1ull) // exponents within a few of each other
                bx = (bx & 0x807fffffu) | ((((by >> 23) & 0xffu) + ((bx >> 23) & 7u) - 3u) & 0xffu) << 23;
            if ((idx & 6ull) == 2ull) // ties of magnitude: the diagonals
                bx = (bx & 0x80000000u) | (by & 0x7fffffffu);
            const float y = __uint_as_float(by), x = __uint_as_float(bx);
            ok = lpm::ff_atan2f(y, x, &f);
            if (ok)
                want = lpm::cr_atan2f_fp64(y, x);
        }
        if (!ok)
            ++und;
        else
        {
            ++dec;
            if (__float_as_uint(f) != __float_as_uint(want))
            {
                ++bad;
                atomicMin(first_bad, idx);
            }
        }
    }
    dec = __reduce_add_sync(0xffffffffu, static_cast<uint32_t>(dec));
    und = __reduce_add_sync(0xffffffffu, static_cast<uint32_t>(und));
    bad = __reduce_add_sync(0xffffffffu, static_cast<uint32_t>(bad));
    if (lane_id() == 0)
    {
        atomicAdd(&stats[0], dec);
        atomicAdd(&stats[1], und);
        atomicAdd(&stats[2], bad);
    }
}

void launch_debug_math_sweep(Launcher& L, int kind, unsigned long long first, unsigned long long count,
                             unsigned long long* stats, unsigned long long* first_bad)
{
    LP_LAUNCH(L, k_debug_math_sweep, 152u * 16u, 256, kind, first, count, stats, first_bad);
}

void launch_segmentation(Launcher& L, const BatchDev& b, const BatchHost& hb, uint8_t* d_image)
{
    const uint32_t T = 256;
    if (hb.any_compute_ring)
        launch_ring_only(L, b, hb);
    LP_LAUNCH(L, k_bin, div_up(b.npts, 2u * T), T, b);
    L.scan(b.cell_cnt, b.cell_start, b.ncell + 1);
    LP_LAUNCH(L, k_scatter, div_up(b.npts, T), T, b);
    LP_LAUNCH(L, k_cell_small, std::min(div_up(b.ncell, 256u), static_cast<uint32_t>(sm_count()) * hb.cell_ctas_per_sm), 256, b);
    LP_LAUNCH(L, k_cell_large, static_cast<uint32_t>(sm_count()) * 2u, 512, b);
    LP_LAUNCH(L, k_chain, div_up(hb.nslices, 128u), 128, b, hb.nslices);
    LP_LAUNCH(L, k_near, div_up(b.nnear * 32u, 256u), 256, b, 0);
    L.scan(b.near_cnt, b.near_start, b.nnear + 1); // near_cnt[nnear] == 0: last entry is the total
    LP_LAUNCH(L, k_near, div_up(b.nnear * 32u, 256u), 256, b, 1);
    LP_LAUNCH(L, k_ransac_draw, static_cast<uint32_t>(b.nscan), 32, b);
    // about four CTAs per SM over the batch's tiles
    LP_LAUNCH(L, k_ransac_inliers, static_cast<uint32_t>(sm_count()) * 4u, 256, b);
    LP_LAUNCH(L, k_ransac_select, div_up(static_cast<uint32_t>(b.nscan), 64u), 64, b);
    LP_LAUNCH(L, k_label_depth, div_up(b.npts, T), T, b);
    LP_LAUNCH(L, k_project_key, div_up(b.npts, T), T, b);
    LP_LAUNCH(L, k_pixel, div_up(b.npix, T), T, b);
    LP_LAUNCH(L, k_dilate_rows, b.nrows, 256, b);
    LP_LAUNCH(L, k_jcp_weights, static_cast<uint32_t>(sm_count()) * hb.jcp_ctas_per_sm, 256, b);
    LP_LAUNCH(L, k_jcp_rowrec, div_up(b.nrows * 32u, 256u), 256, b);
    LP_LAUNCH_SMEM(L, k_jcp_rows, static_cast<uint32_t>(b.nscan), 256, 2u * kStageBytes, b);
    LP_LAUNCH(L, k_populate, div_up(b.npix, T), T, b, d_image);
}
} // namespace lpg
