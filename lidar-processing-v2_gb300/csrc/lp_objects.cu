// lp_objects.cu — the processor's per-cluster products after the hulls (Processor::run,
// processor.cpp:609-797): the clustered cloud, the boundary marker geometry, and (lp_hull.cu,
// k_obj_gate) the vehicle gates.
//
// Clustered cloud (processor.cpp:627-658): the reference visits labels 0..K-1 and, for each, every
// obstacle point in input order, so the cloud is a stable grouping of the clustered points by
// label. Here a counting sort: per 8,192-point tile and label a count (label-major matrix), one
// exclusive scan of the matrix gives every (label, tile) its first slot, and one warp per tile
// places the tile's points in order (lanes with the same label ranked by __match_any_sync). The
// colours are std::rand() % 256 for r, g, b per label, in label order; the stream is glibc's
// additive feedback generator, whose 34-value window the host positions at the scan's first draw
// (the stream's offset is a caller input), and one thread draws the 3K values.
//
// Markers (convertPolygonPointsToMarker, processor.cpp:241-343): per cluster with a polygon of at
// least 3 points (the gate's box corners for a classified cluster, else the hull vertices in hull
// order), the LINE_LIST points of the bottom ring at z_min, the top ring at z_max and the vertical
// edges: 6 per vertex, counted, scanned and written per cluster.
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
constexpr uint32_t kObjTile = 8192;

__global__ void k_obj_hist(const int32_t* labels, uint32_t n, uint32_t K, uint32_t ntiles, uint32_t* cnt, uint32_t* err)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const int32_t l = (i < n) ? labels[i] : -1;
    const bool bad = l >= 0 && static_cast<uint32_t>(l) >= K;
    if (bad)
        atomicOr(err, 1u);
    const int32_t key = (l >= 0 && !bad) ? l : -1;
    // lanes of a warp share a tile (the tile is a multiple of 32 points): one add per label
    const uint32_t same = __match_any_sync(0xffffffffu, key);
    if (key >= 0 && lane_id() == static_cast<uint32_t>(__ffs(static_cast<int>(same)) - 1))
        atomicAdd(&cnt[static_cast<size_t>(key) * ntiles + i / kObjTile], static_cast<uint32_t>(__popc(same)));
}

// First cloud slot of each label (the scanned matrix's label-major row starts), and the total.
__global__ void k_obj_offsets(const uint32_t* start, uint32_t K, uint32_t ntiles, uint32_t* cl_off)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l <= K)
        cl_off[l] = start[static_cast<size_t>(l) * ntiles];
}

// glibc rand() from the window the host positioned (34 values, `pos` = slot of the next value):
// r[i] = r[i-31] + r[i-3] mod 2^32, output r[i] >> 1; colours r, g, b = three outputs % 256.
__global__ void k_obj_colors(RandWindow w, uint32_t K, uchar4* colour)
{
    if (blockIdx.x != 0 || threadIdx.x != 0)
        return;
    uint32_t pos = w.pos;
    auto next = [&]() -> uint32_t {
        const uint32_t v = w.r[(pos + 3u) % 34u] + w.r[(pos + 31u) % 34u];
        w.r[pos] = v;
        pos = (pos + 1u) % 34u;
        return (v >> 1) % 256u;
    };
    for (uint32_t l = 0; l < K; ++l)
    {
        const uint32_t r = next(), g = next(), b = next();
        colour[l] = make_uchar4(static_cast<unsigned char>(r), static_cast<unsigned char>(g),
                                static_cast<unsigned char>(b), 255);
    }
}

// One warp per tile, the tile's points in order: rank among the 32-point step's lanes of the same
// label plus the (label, tile) running slot, which only this warp advances.
__global__ void k_obj_place(const float4* pts, const int32_t* labels, uint32_t n, uint32_t K, uint32_t ntiles,
                            uint32_t* run, const uchar4* colour, lp_xyzrgb* cloud)
{
    const uint32_t t = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    if (t >= ntiles)
        return;
    const uint32_t lane = lane_id();
    const uint32_t below = (1u << lane) - 1u;
    const uint32_t end = min(n, (t + 1) * kObjTile);
    for (uint32_t base = t * kObjTile; base < end; base += 32)
    {
        const uint32_t i = base + lane;
        const int32_t l = (i < end) ? labels[i] : -1;
        const int32_t key = (l >= 0 && static_cast<uint32_t>(l) < K) ? l : -1;
        const uint32_t same = __match_any_sync(0xffffffffu, key);
        const uint32_t leader = static_cast<uint32_t>(__ffs(static_cast<int>(same)) - 1);
        uint32_t slot = 0;
        if (key >= 0 && lane == leader)
        {
            uint32_t* r = &run[static_cast<size_t>(key) * ntiles + t];
            slot = *r;
            *r = slot + static_cast<uint32_t>(__popc(same));
        }
        slot = __shfl_sync(0xffffffffu, slot, leader);
        if (key >= 0)
        {
            const float4 p = pts[i];
            const uchar4 c = colour[key];
            cloud[slot + __popc(same & below)] = lp_xyzrgb{p.x, p.y, p.z, c.x, c.y, c.z, c.w};
        }
        __syncwarp();
    }
}

// Polygon of a cluster: the gate's box corners when it classified the cluster, else the hull.
__device__ __forceinline__ uint32_t obj_polygon_size(const ObjDev& o, uint32_t l)
{
    return (o.cls[l] >= 0) ? 4u : o.hull_off[l + 1] - o.hull_off[l];
}

__device__ __forceinline__ double2 obj_polygon_point(const ObjDev& o, uint32_t l, uint32_t k)
{
    if (o.cls[l] >= 0)
        return make_double2(o.boxes[l].corners[k][0], o.boxes[l].corners[k][1]);
    const lp_xyzrgb& p = o.cloud[o.cl_off[l] + static_cast<uint32_t>(o.hull_idx[o.hull_off[l] + k])];
    return make_double2(static_cast<double>(p.x), static_cast<double>(p.y));
}

__global__ void k_obj_marker_count(ObjDev o)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > o.K)
        return;
    const uint32_t m = (l < o.K) ? obj_polygon_size(o, l) : 0u;
    o.moff[l] = (m >= 3u) ? 6u * m : 0u;
}

__global__ void k_obj_marker_write(ObjDev o)
{
    const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= o.K)
        return;
    const uint32_t m = obj_polygon_size(o, l);
    uint32_t at = o.moff[l];
    if (m < 3u || at + 6u * m > o.mcap)
        return;
    const double zlo = static_cast<double>(o.zmin[l]), zhi = static_cast<double>(o.zmax[l]);
    auto put = [&](double2 p, double z) {
        o.mpts[3ull * at] = p.x;
        o.mpts[3ull * at + 1] = p.y;
        o.mpts[3ull * at + 2] = z;
        ++at;
    };
    for (int ring = 0; ring < 2; ++ring)
    {
        const double z = ring ? zhi : zlo;
        for (uint32_t k = 1; k < m; ++k)
        {
            put(obj_polygon_point(o, l, k - 1), z);
            put(obj_polygon_point(o, l, k), z);
        }
        put(obj_polygon_point(o, l, m - 1), z);
        put(obj_polygon_point(o, l, 0), z);
    }
    for (uint32_t k = 0; k < m; ++k)
    {
        const double2 p = obj_polygon_point(o, l, k);
        put(p, zlo);
        put(p, zhi);
    }
}
} // namespace

uint32_t obj_tiles(uint32_t n)
{
    return div_up(std::max(n, 1u), kObjTile);
}

void launch_objects_cloud(cudaStream_t st, const float4* pts, const int32_t* labels, uint32_t n, uint32_t K,
                          uint32_t* cnt, uint32_t* sums, uint32_t* err, const RandWindow& w, uchar4* colour,
                          uint32_t* cl_off, lp_xyzrgb* cloud, uint64_t& launches)
{
    const uint32_t ntiles = obj_tiles(n);
    const uint32_t cells = K * ntiles + 1;
    k_obj_hist<<<div_up(std::max(n, 1u), 256u), 256, 0, st>>>(labels, n, K, ntiles, cnt, err);
    scan_exclusive(st, cnt, cnt, cells, sums, nullptr, launches);
    k_obj_offsets<<<div_up(K + 1, 256u), 256, 0, st>>>(cnt, K, ntiles, cl_off);
    k_obj_colors<<<1, 1, 0, st>>>(w, K, colour);
    k_obj_place<<<div_up(ntiles, 4u), 128, 0, st>>>(pts, labels, n, K, ntiles, cnt, colour, cloud);
    launches += 5;
}

void launch_objects_markers(cudaStream_t st, const ObjDev& o, uint32_t* sums, uint64_t& launches)
{
    k_obj_marker_count<<<div_up(o.K + 1, 256u), 256, 0, st>>>(o);
    scan_exclusive(st, o.moff, o.moff, o.K + 1, sums, nullptr, launches);
    k_obj_marker_write<<<div_up(std::max(o.K, 1u), 128u), 128, 0, st>>>(o);
    launches += 2;
}
} // namespace lpg
