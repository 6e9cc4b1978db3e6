// lp_internal.cuh — batch layout shared by the kernels of liblp_gpu.so.
//
// A batch is S scans laid out back to back in device memory (HBM). Every per-point, per-pixel,
// per-cell array of the batch is one flat array; a scan owns the slice [off, off + count) of
// each, recorded in its ScanDev descriptor. A single scan is a batch of one, so the plain
// (one scan per launch sequence) and the batched form run the same kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lidar_gb300.h"

namespace lpg
{
constexpr int kMaxRansacIters = 60;  // segmenter.cpp:324
constexpr int kRansacRadialBins = 4; // segmenter.cpp:323
constexpr uint32_t kVoxelCapacity = 200000u; // clusterer.cpp:36 (StaticUnorderedMap reserve)

// Error bits raised by kernels in ScanState::err (read back with the results).
enum : uint32_t
{
    ERR_CELL_TOO_LARGE = 1u << 0,
    ERR_VOXEL_CAPACITY = 1u << 1,
    ERR_HASH_FULL = 1u << 2,
    ERR_HULL_CAPACITY = 1u << 3,
    ERR_CLUSTER_CAPACITY = 1u << 4,
    ERR_UF_TIMEOUT = 1u << 5,
    ERR_INTERNAL = 1u << 6,
};

// Static per-scan description: sizes, offsets into the batch arrays and configuration values
// precomputed on the host with the same binary32 expressions the reference evaluates.
struct ScanDev
{
    // points (after optional noise compaction)
    uint32_t pt_off, n;
    uint32_t src_off, n_src; // original input points (before noise compaction)
    // range image
    uint32_t pix_off;
    int32_t H, W;
    uint32_t row_off;   // first global row (sum of H of earlier scans)
    uint32_t tile_off;  // first 1024-point ring tile
    uint32_t slice_off; // first global azimuth slice
    // polar grid
    uint32_t cell_off;
    int32_t nslice, nrad;
    uint32_t near_off; // near-field cells (radial < 4), nslice * min(4, nrad)
    int32_t nnear_per_slice;
    // segmentation constants (segmenter.cpp:106-122, :209-211, :360)
    float zmin_adj, zmax_adj, spacing, min_d, max_d, slice_res;
    float down_rad, rad_per_px;
    float delta, thr, sensor_h, kthr2, amp, max_cos;
    int32_t use_ring; // 1: height index from ring; 0: from the elevation angle
    int32_t compute_ring;
    int32_t first_ring;
    // clustering constants (clusterer.hpp:76-90)
    float res_r, res_a, res_e;
    uint32_t min_cluster;
    uint32_t hash_off, hash_cap; // voxel hash table slice (power of two)
    // per-cluster output capacity
    uint32_t cluster_cap, hull_cap;
    uint32_t cl_off; // offset of this scan's cluster arrays
    uint32_t hull_off;
    // DROR (noise_remover.cpp:49-57): s2 = pow(double(multiplier), 2), rmin2 = rmin * rmin
    double dror_s2;
    float dror_rmin2;
    uint32_t dror_k;
};

// Dynamic per-scan values produced on the device.
struct ScanState
{
    uint32_t err;
    uint32_t n_pts;     // points entering segmentation (after noise removal)
    uint32_t reserved_dror[2];
    // RANSAC (segmenter.cpp:321-479)
    uint32_t n_cand, cand_off;
    int32_t ransac_ok;
    float plane[4];
    // clustering
    uint32_t n_obs, obs_off;
    uint32_t max_r_bits, max_a_bits, max_e_bits;
    int32_t nr, na, ne;
    uint32_t n_vox;
    uint32_t n_comp;
    uint32_t n_clusters;
    uint32_t cl_base; // clusters of earlier scans (work-queue numbering)
    uint32_t n_hull;
    uint32_t pad[4];
};

__device__ __forceinline__ void raise_err(ScanState* st, uint32_t bit)
{
    atomicOr(&st->err, bit);
}

// Binary search of the scan that owns flat index `i` given ascending offsets.
template <typename F>
__device__ __forceinline__ int find_scan(int nscan, uint32_t i, F off_of)
{
    int lo = 0, hi = nscan - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        if (off_of(mid) <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Order-preserving map of non-negative float bits for atomicMax.
__device__ __forceinline__ uint32_t fkey(float v)
{
    return __float_as_uint(v);
}

__device__ __forceinline__ uint32_t lane_id()
{
    return threadIdx.x & 31u;
}

// Kernel launch bookkeeping (counted by the host wrapper for instrumentation).
struct LaunchCounter
{
    uint64_t n = 0;
};

} // namespace lpg
