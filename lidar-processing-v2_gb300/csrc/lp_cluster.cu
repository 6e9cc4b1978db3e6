// lp_cluster.cu — curved-voxel clustering of the obstacle points.
//
// Reference: lidar_processing_lib/src/clusterer.cpp. The reference labels 26-connected
// components of occupied (range, azimuth, elevation) voxels by a BFS seeded in point order, so
// a component's label is the rank of its smallest point index; components smaller than
// min_cluster_size are dropped and the rest renumbered in the same order (clusterer.cpp:
// 122-239). Here: a per-scan open-addressing hash of occupied voxels, lock-free union-find over
// the 26-neighbour graph (the azimuth index wraps modulo num_azimuth as in clusterer.cpp:
// 161-169), and the canonical labels from a prefix scan of "component minimum" flags. Labels
// are identical to the reference's, not only the partition.
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_math.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
constexpr float kTwoPiF = 6.28318548202514648438f; // Clusterer::TWO_M_PIf
constexpr float kPi2F = 1.57079637050628662109f;   // M_PI_2f
constexpr uint32_t kEmpty = 0xffffffffu;
constexpr int kMaxIters = 1 << 22;

__device__ __forceinline__ int scan_of_obs(const BatchDev& b, uint32_t o)
{
    return find_scan(b.nscan, o, [&](int s) { return b.state[s].obs_off; });
}
__device__ __forceinline__ int scan_of_hash(const BatchDev& b, uint32_t h)
{
    return find_scan(b.nscan, h, [&](int s) { return b.scans[s].hash_off; });
}
__device__ __forceinline__ uint32_t hash_mix(uint32_t k)
{
    k *= 0x9E3779B1u;
    k ^= k >> 15;
    k *= 0x85EBCA77u;
    k ^= k >> 13;
    return k;
}
__device__ __forceinline__ uint32_t ld_volatile(const uint32_t* p)
{
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

__global__ void k_obs_flag(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > b.npts)
        return;
    b.obs_flag[i] = (i < b.npts && b.seg_label[i] == LP_LABEL_OBSTACLE) ? 1u : 0u;
}

__global__ void k_obs_state(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    st.obs_off = b.obs_flag[sd.pt_off];
    st.n_obs = b.obs_flag[sd.pt_off + sd.n] - st.obs_off;
    st.max_r_bits = 0u;
    st.max_a_bits = 0u;
    st.max_e_bits = 0u;
}

// Obstacle cloud in input order (processor.cpp:562-579) with the spherical coordinates of
// Clusterer::cartesianToSpherical (clusterer.cpp:55-100). A block takes 1024 consecutive points
// and first compacts its obstacle points in shared memory, so that every lane of the arithmetic
// below (two correctly rounded arctangents) has one.
constexpr uint32_t kObsChunk = 1024;

__global__ void __launch_bounds__(256) k_obs_gather(BatchDev b)
{
    __shared__ uint32_t sidx[kObsChunk];
    __shared__ uint32_t scnt;
    const uint32_t base = blockIdx.x * kObsChunk;
    if (threadIdx.x == 0)
        scnt = 0u;
    __syncthreads();
#pragma unroll
    for (uint32_t u = 0; u < kObsChunk / 256u; ++u)
    {
        const uint32_t i = base + u * 256u + threadIdx.x;
        const bool valid = i < b.npts && b.seg_label[i] == LP_LABEL_OBSTACLE;
        const uint32_t m = __ballot_sync(0xffffffffu, valid);
        uint32_t pos = 0u;
        if (lane_id() == 0 && m)
            pos = atomicAdd(&scnt, static_cast<uint32_t>(__popc(m)));
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (valid)
            sidx[pos + static_cast<uint32_t>(__popc(m & ((1u << lane_id()) - 1u)))] = i;
    }
    __syncthreads();
    const uint32_t cnt = scnt;
    for (uint32_t k0 = 0; k0 < cnt; k0 += 256u)
    {
        const uint32_t k = k0 + threadIdx.x;
        const bool valid = k < cnt;
        const uint32_t i = valid ? sidx[k] : 0u;
        const int s = valid ? scan_of_point(b, i) : -1;
        uint32_t rb = 0u, ab = 0u, eb = 0u;
        if (valid)
        {
            const uint32_t o = b.obs_flag[i];
            const float4 p = b.pts[i];
            b.obs_pts[o] = p;
            b.obs_pt[o] = static_cast<int32_t>(i);
            float az = lpm::cr_atan2f(p.y, p.x);
            az = (az < 0) ? (az + kTwoPiF) : az;
            const float d2 = p.x * p.x + p.y * p.y;
            const float d = sqrtf(d2);
            const float r = sqrtf(d2 + p.z * p.z);
            const float el = lpm::cr_atanf(p.z / d) + kPi2F;
            b.obs_r[o] = r;
            b.obs_a[o] = az;
            b.obs_e[o] = el;
            rb = r > 0.0f ? __float_as_uint(r) : 0u; // non-negative floats order like their bits
            ab = az > 0.0f ? __float_as_uint(az) : 0u;
            eb = el > 0.0f ? __float_as_uint(el) : 0u;
        }
        // one atomic per warp when the warp's obstacle points belong to a single scan
        const int smax = static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<unsigned>(s + 1))) - 1;
        if (__all_sync(0xffffffffu, s == smax || s < 0))
        {
            rb = __reduce_max_sync(0xffffffffu, rb);
            ab = __reduce_max_sync(0xffffffffu, ab);
            eb = __reduce_max_sync(0xffffffffu, eb);
            if (lane_id() == 0 && smax >= 0)
            {
                ScanState& st = b.state[smax];
                atomicMax(&st.max_r_bits, rb);
                atomicMax(&st.max_a_bits, ab);
                atomicMax(&st.max_e_bits, eb);
            }
        }
        else if (valid)
        {
            ScanState& st = b.state[s];
            atomicMax(&st.max_r_bits, rb);
            atomicMax(&st.max_a_bits, ab);
            atomicMax(&st.max_e_bits, eb);
        }
    }
}

__global__ void k_dims(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    if (st.n_obs == 0)
    {
        st.nr = st.na = st.ne = 0;
        return;
    }
    st.nr = static_cast<int32_t>(ceilf(__uint_as_float(st.max_r_bits) / sd.res_r) + 1.0f);
    st.na = static_cast<int32_t>(ceilf(__uint_as_float(st.max_a_bits) / sd.res_a) + 1.0f);
    st.ne = static_cast<int32_t>(ceilf(__uint_as_float(st.max_e_bits) / sd.res_e) + 1.0f);
    const long long cells = static_cast<long long>(st.nr) * st.na * st.ne;
    if (cells > 0x7fffffffLL)
        raise_err(&st, ERR_INTERNAL);
}

__device__ __forceinline__ int32_t flat_voxel(int32_t nr, int32_t na, int32_t r, int32_t a, int32_t e)
{
    return nr * (na * e + a) + r; // Clusterer::flatVoxelIndex, clusterer.hpp:136-142
}

__global__ void k_vox_insert(BatchDev b)
{
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= b.obs_flag[b.npts])
        return;
    const int s = scan_of_obs(b, o);
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    const int32_t vr = static_cast<int32_t>(b.obs_r[o] / sd.res_r);
    const int32_t va = static_cast<int32_t>(b.obs_a[o] / sd.res_a);
    const int32_t ve = static_cast<int32_t>(b.obs_e[o] / sd.res_e);
    const uint32_t key = static_cast<uint32_t>(flat_voxel(st.nr, st.na, vr, va, ve));
    const uint32_t mask = sd.hash_cap - 1u;
    uint32_t h = hash_mix(key) & mask;
    for (uint32_t probe = 0; probe < sd.hash_cap; ++probe)
    {
        const uint32_t slot = sd.hash_off + h;
        const uint32_t prev = atomicCAS(&b.hkey[slot], kEmpty, key);
        if (prev == kEmpty || prev == key)
        {
            b.obs_hslot[o] = slot;
            atomicMin(&b.hmin[slot], o - st.obs_off);
            atomicAdd(&b.hcnt[slot], 1u);
            return;
        }
        h = (h + 1u) & mask;
    }
    raise_err(&st, ERR_HASH_FULL);
    b.obs_hslot[o] = kEmpty;
}

// Voxel ids in hash-slot order: one look-back scan reads the occupancy of the hash slots, writes
// hvid[h] = the number of occupied slots before h (nhash + 1 entries: the last is the total) and
// initialises the union-find record of every occupied slot's voxel.
struct VoxFlagsSrc
{
    const uint32_t* hkey;
    uint32_t nhash;
    __device__ __forceinline__ uint4 get4(uint32_t i) const
    {
        uint4 k;
        if (i + 4u <= nhash)
            k = *reinterpret_cast<const uint4*>(hkey + i);
        else
        {
            k.x = (i < nhash) ? hkey[i] : kEmpty;
            k.y = (i + 1u < nhash) ? hkey[i + 1u] : kEmpty;
            k.z = (i + 2u < nhash) ? hkey[i + 2u] : kEmpty;
            k.w = (i + 3u < nhash) ? hkey[i + 3u] : kEmpty;
        }
        return make_uint4(k.x != kEmpty, k.y != kEmpty, k.z != kEmpty, k.w != kEmpty);
    }
};
struct VoxInitDst
{
    uint32_t *hvid, *vslot, *parent, *cmin, *ccnt;
    uint32_t n; // nhash + 1
    __device__ __forceinline__ void one(uint32_t h, uint32_t v, uint32_t occupied) const
    {
        if (occupied)
        {
            vslot[v] = h;
            parent[v] = v;
            cmin[v] = kEmpty;
            ccnt[v] = 0u;
        }
    }
    __device__ __forceinline__ void put4(uint32_t i, uint4 e, uint4 f) const
    {
        ScanDstU32{hvid, n, true}.put4(i, e, f);
        one(i, e.x, f.x);
        one(i + 1u, e.y, f.y);
        one(i + 2u, e.z, f.z);
        one(i + 3u, e.w, f.w);
    }
};

__global__ void k_vox_count(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    st.n_vox = b.hvid[sd.hash_off + sd.hash_cap] - b.hvid[sd.hash_off];
    if (st.n_vox > kVoxelCapacity)
        raise_err(&st, ERR_VOXEL_CAPACITY); // StaticUnorderedMap::insert throws (static_unordered_map.hpp:81)
}

// Every parent pointer is strictly smaller than its index except at roots (links go from the
// larger root to the smaller; path halving only shortens), so a find ends within x steps. The
// per-thread budget bounds the total work anyway: exhausting it raises ERR_UF_TIMEOUT.
__device__ uint32_t uf_find(uint32_t* parent, uint32_t x, ScanState* st, int& budget)
{
    while (budget-- > 0)
    {
        const uint32_t p = ld_volatile(&parent[x]);
        if (p == x)
            return x;
        const uint32_t gp = ld_volatile(&parent[p]);
        if (gp != p)
            atomicCAS(&parent[x], p, gp); // path halving; parents only ever decrease
        x = gp;
    }
    raise_err(st, ERR_UF_TIMEOUT);
    return x;
}

__device__ void uf_union(uint32_t* parent, uint32_t a, uint32_t c, ScanState* st, int& budget)
{
    while (budget > 0)
    {
        a = uf_find(parent, a, st, budget);
        c = uf_find(parent, c, st, budget);
        if (budget <= 0)
            return;
        if (a == c)
            return;
        if (a > c)
        {
            const uint32_t t = a;
            a = c;
            c = t;
        }
        // link the larger root below the smaller one
        const uint32_t old = atomicCAS(&parent[c], c, a);
        if (old == c)
            return;
        c = old;
    }
    raise_err(st, ERR_UF_TIMEOUT);
}

__device__ __forceinline__ uint32_t hash_lookup(const BatchDev& b, const ScanDev& sd, uint32_t key)
{
    const uint32_t mask = sd.hash_cap - 1u;
    uint32_t h = hash_mix(key) & mask;
    for (uint32_t probe = 0; probe < sd.hash_cap; ++probe)
    {
        const uint32_t k = b.hkey[sd.hash_off + h];
        if (k == key)
            return sd.hash_off + h;
        if (k == kEmpty)
            return kEmpty;
        h = (h + 1u) & mask;
    }
    return kEmpty;
}

// Neighbour offsets (clusterer.hpp:101-105): all 26 (dr, da, de) != (0, 0, 0). Only the 13 after
// (0, 0, 0) in (de, da, dr) order are probed: every adjacent pair of voxels is then met from one
// side (or both, where the azimuth wraps onto itself), which yields the same components as probing
// all 26. One (voxel, offset) pair per thread: the probes are chains of dependent loads, so they
// run side by side; the components (and the labels, component minima) do not depend on the order
// of the unions.
__device__ __forceinline__ void k_uf_hook_pair(const BatchDev& b, uint32_t v, uint32_t o)
{
    // offset o: 0 -> (de 0, da 0, dr +1), 1..3 -> (0, +1, -1..+1), 4..12 -> (+1, -1..+1, -1..+1)
    const int32_t de = (o < 4u) ? 0 : 1;
    const int32_t da = (o == 0u) ? 0 : ((o < 4u) ? 1 : static_cast<int32_t>((o - 4u) / 3u) - 1);
    const int32_t dr = (o == 0u) ? 1 : ((o < 4u) ? static_cast<int32_t>(o) - 2 : static_cast<int32_t>((o - 4u) % 3u) - 1);
    const uint32_t slot = b.vslot[v];
    const int s = scan_of_hash(b, slot);
    const ScanDev& sd = b.scans[s];
    ScanState* st = &b.state[s];
    const int32_t nr = st->nr, na = st->na, ne = st->ne;
    const int32_t key = static_cast<int32_t>(b.hkey[slot]);
    const int32_t r = key % nr;
    const int32_t a = (key / nr) % na;
    const int32_t e = key / (nr * na);
    const int32_t rr = r + dr, ee = e + de;
    if (rr < 0 || rr >= nr || ee < 0 || ee >= ne)
        return;
    int32_t aa = a + da;
    if (aa < 0)
        aa += na;
    else if (aa >= na)
        aa -= na;
    const uint32_t nslot = hash_lookup(b, sd, static_cast<uint32_t>(flat_voxel(nr, na, rr, aa, ee)));
    if (nslot == kEmpty)
        return;
    const uint32_t u = b.hvid[nslot];
    if (u != v)
    {
        int budget = kMaxIters;
        uf_union(b.parent, v, u, st, budget);
    }
}

__global__ void k_uf_hook(BatchDev b)
{
    const uint32_t nv = b.hvid[b.nhash]; // occupied voxels; threads stride over (offset, voxel) pairs
    const unsigned long long total = 13ull * nv;
    for (unsigned long long t = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; t < total;
         t += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
        k_uf_hook_pair(b, static_cast<uint32_t>(t % nv), static_cast<uint32_t>(t / nv));
}

__device__ __forceinline__ void k_uf_flatten_one(const BatchDev& b, uint32_t v)
{
    const uint32_t slot = b.vslot[v];
    const int s = scan_of_hash(b, slot);
    int budget = kMaxIters;
    const uint32_t root = uf_find(b.parent, v, &b.state[s], budget);
    b.parent[v] = root;
}

__global__ void k_uf_flatten(BatchDev b)
{
    const uint32_t nv = b.hvid[b.nhash]; // occupied voxels: persistent threads stride over them
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        k_uf_flatten_one(b, v);
}

__device__ __forceinline__ void k_comp_stats_one(const BatchDev& b, uint32_t v)
{
    const uint32_t root = b.parent[v];
    const uint32_t slot = b.vslot[v];
    atomicMin(&b.cmin[root], b.hmin[slot]);
    atomicAdd(&b.ccnt[root], b.hcnt[slot]);
}

__global__ void k_comp_stats(BatchDev b)
{
    const uint32_t nv = b.hvid[b.nhash]; // occupied voxels: persistent threads stride over them
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        k_comp_stats_one(b, v);
}

__device__ __forceinline__ void k_keep_one(const BatchDev& b, uint32_t v)
{
    if (b.parent[v] != v)
        return;
    const uint32_t slot = b.vslot[v];
    const int s = scan_of_hash(b, slot);
    if (b.ccnt[v] >= b.scans[s].min_cluster)
        b.kflag[b.state[s].obs_off + b.cmin[v]] = 1u;
}

__global__ void k_keep(BatchDev b)
{
    const uint32_t nv = b.hvid[b.nhash];
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        k_keep_one(b, v);
}

// kflag now holds the exclusive scan: rank of each kept component among the scan's kept
// components ordered by smallest point index == the reference's final label.
__global__ void k_obs_label(BatchDev b)
{
    __shared__ BlockAgg agg;
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    const bool in = o < b.obs_flag[b.npts];
    int32_t label = LP_INVALID_CLUSTER;
    uint32_t g = 0u;
    if (in)
    {
        const int s = scan_of_obs(b, o);
        const ScanDev& sd = b.scans[s];
        const ScanState& st = b.state[s];
        const uint32_t slot = b.obs_hslot[o];
        if (slot != kEmpty)
        {
            const uint32_t root = b.parent[b.hvid[slot]];
            if (b.ccnt[root] >= sd.min_cluster)
                label = static_cast<int32_t>(b.kflag[st.obs_off + b.cmin[root]] - b.kflag[st.obs_off]);
        }
        b.obs_label[o] = label;
        g = sd.cl_off + static_cast<uint32_t>(label);
    }
    block_aggregated_inc(b.cl_cnt, g, in && label >= 0, agg);
}

__global__ void k_cl_state(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    st.n_clusters = b.kflag[st.obs_off + st.n_obs] - b.kflag[st.obs_off];
    if (st.n_clusters > sd.cluster_cap)
        raise_err(&st, ERR_CLUSTER_CAPACITY);
}

// Members grouped by cluster (slot order within a cluster is free), with their x, y alongside for
// the hull stage, and each cluster's z range (ordered-key maxima: one atomic pair per cluster and
// warp where a warp's points share few clusters; otherwise per point, skipped when a fresh read
// of the key shows it cannot rise).
__device__ __forceinline__ uint32_t z_ord(float f)
{
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void k_cl_scatter(BatchDev b)
{
    __shared__ BlockAgg agg;
    const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t lane = lane_id();
    const int32_t label = (o < b.obs_flag[b.npts]) ? b.obs_label[o] : -1;
    const bool in = label >= 0;
    uint32_t g = 0u;
    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
    if (in)
    {
        g = b.scans[scan_of_obs(b, o)].cl_off + static_cast<uint32_t>(label);
        p = b.obs_pts[o];
    }
    const uint32_t rank = block_aggregated_inc(b.cl_fill, g, in, agg);
    if (in)
    {
        const uint32_t slot = b.cl_start[g] + rank;
        b.members[slot] = o;
        b.mxy[slot] = make_float2(p.x, p.y);
    }
    const uint32_t zo = z_ord(p.z);
    const uint32_t peers = __match_any_sync(0xffffffffu, in ? g : 0xffffffffu);
    const uint32_t groups = __popc(__ballot_sync(0xffffffffu, in && lane == static_cast<uint32_t>(__ffs(peers) - 1)));
    if (groups > 4u)
    {
        if (in)
        {
            if (~zo > __ldcg(&b.cl_zkey[2u * g]))
                atomicMax(&b.cl_zkey[2u * g], ~zo);
            if (zo > __ldcg(&b.cl_zkey[2u * g + 1u]))
                atomicMax(&b.cl_zkey[2u * g + 1u], zo);
        }
        return;
    }
    for (uint32_t todo = __ballot_sync(0xffffffffu, in); todo != 0u;)
    {
        const int l = __ffs(todo) - 1;
        const uint32_t lg = __shfl_sync(0xffffffffu, g, l);
        const bool mine = in && g == lg;
        const uint32_t lo = __reduce_max_sync(0xffffffffu, mine ? ~zo : 0u);
        const uint32_t hi = __reduce_max_sync(0xffffffffu, mine ? zo : 0u);
        if (lane == static_cast<uint32_t>(l))
        {
            atomicMax(&b.cl_zkey[2u * lg], lo);
            atomicMax(&b.cl_zkey[2u * lg + 1u], hi);
        }
        todo &= ~__ballot_sync(0xffffffffu, mine);
    }
}
} // namespace

// Clusterer::cluster on a caller-supplied cloud: every point is a member of the cloud to cluster.
__global__ void k_mark_all(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.npts)
        return;
    const int s = scan_of_point(b, i);
    b.seg_label[i] = (i - b.scans[s].pt_off < b.state[s].n_pts) ? LP_LABEL_OBSTACLE : LP_LABEL_UNKNOWN;
}

void launch_mark_all_obstacles(Launcher& L, const BatchDev& b)
{
    LP_LAUNCH(L, k_mark_all, div_up(b.npts, 256u), 256, b);
}

void launch_clustering(Launcher& L, const BatchDev& b, const BatchHost& hb)
{
    const uint32_t T = 256;
    const uint32_t ns = static_cast<uint32_t>(b.nscan);
    LP_LAUNCH(L, k_obs_flag, div_up(b.npts + 1, T), T, b);
    L.scan(b.obs_flag, b.obs_flag, b.npts + 1);
    LP_LAUNCH(L, k_obs_state, div_up(ns, 64u), 64, b);
    LP_LAUNCH(L, k_obs_gather, div_up(b.npts, kObsChunk), 256, b);
    LP_LAUNCH(L, k_dims, div_up(ns, 64u), 64, b);
    LP_LAUNCH(L, k_vox_insert, div_up(b.npts, T), T, b);
    L.begin("k_vox_ids");
    scan_lookback(L.stream, VoxFlagsSrc{b.hkey, b.nhash}, VoxInitDst{b.hvid, b.vslot, b.parent, b.cmin, b.ccnt, b.nhash + 1},
                  b.nhash + 1, L.scan_sums, L.scan_err);
    L.end();
    L.note();
    LP_LAUNCH(L, k_vox_count, div_up(ns, 64u), 64, b);
    const uint32_t vgrid = std::min(div_up(b.nhash, T), static_cast<uint32_t>(sm_count()) * 8u); // <= voxels
    LP_LAUNCH(L, k_uf_hook, vgrid, T, b);
    LP_LAUNCH(L, k_uf_flatten, vgrid, T, b);
    LP_LAUNCH(L, k_comp_stats, vgrid, T, b);
    LP_LAUNCH(L, k_keep, vgrid, T, b);
    L.scan(b.kflag, b.kflag, b.npts + 1);
    LP_LAUNCH(L, k_obs_label, div_up(b.npts, T), T, b);
    LP_LAUNCH(L, k_cl_state, div_up(ns, 64u), 64, b);
    L.scan(b.cl_cnt, b.cl_start, b.ncl + 1);
    LP_LAUNCH(L, k_cl_scatter, div_up(b.npts, T), T, b);
    (void)hb;
}
} // namespace lpg
