// lp_stages.hpp — host-side launch helpers and the stage entry points of liblp_gpu.so.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <string>
#include <vector>

#include "lp_batch.cuh"

namespace lpg
{
void scan_exclusive(cudaStream_t st, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* err,
                    uint64_t& launches);
void launch_debug_wait_timeout(cudaStream_t st, int kind, uint32_t limit, unsigned long long* state, uint32_t* err,
                               uint64_t& launches);

// One timed launch (profiling mode only).
struct LaunchRecord
{
    const char* name;
    cudaEvent_t start, stop;
};

// Issues kernel launches on one stream, counts them and remembers the first launch error. In
// profiling mode every launch is bracketed by CUDA events on the same stream.
struct Launcher
{
    cudaStream_t stream = nullptr;
    uint64_t* launches = nullptr;
    uint32_t* scan_sums = nullptr; // scratch for device-wide scans
    uint32_t* scan_err = nullptr;  // error word the device-wide scans report into
    cudaError_t err = cudaSuccess;
    std::vector<LaunchRecord>* prof = nullptr;
    std::vector<cudaEvent_t>* event_pool = nullptr;
    size_t pool_next = 0;

    cudaEvent_t next_event()
    {
        if (pool_next >= event_pool->size())
        {
            cudaEvent_t e;
            cudaEventCreate(&e);
            event_pool->push_back(e);
        }
        return (*event_pool)[pool_next++];
    }
    void begin(const char* name)
    {
        if (prof)
        {
            LaunchRecord r{name, next_event(), next_event()};
            cudaEventRecord(r.start, stream);
            prof->push_back(r);
        }
    }
    void end()
    {
        if (prof)
            cudaEventRecord(prof->back().stop, stream);
    }

    template <typename K, typename... Args>
    void launch(const char* name, K kernel, uint32_t grid, uint32_t block, Args... args)
    {
        if (grid == 0)
            return;
        begin(name);
        kernel<<<grid, block, 0, stream>>>(args...);
        end();
        note();
    }
    template <typename K, typename... Args>
    void launch2d(const char* name, K kernel, dim3 grid, uint32_t block, Args... args)
    {
        if (grid.x == 0 || grid.y == 0)
            return;
        begin(name);
        kernel<<<grid, block, 0, stream>>>(args...);
        end();
        note();
    }
    template <typename K, typename... Args>
    void launch_smem(const char* name, K kernel, uint32_t grid, uint32_t block, size_t smem, Args... args)
    {
        if (grid == 0)
            return;
        begin(name);
        kernel<<<grid, block, smem, stream>>>(args...);
        end();
        note();
    }
    void scan(const uint32_t* in, uint32_t* out, uint32_t n)
    {
        if (n == 0)
            return;
        begin("k_scan");
        scan_exclusive(stream, in, out, n, scan_sums, scan_err, *launches);
        end();
        note_only();
    }
    void note()
    {
        ++(*launches);
        note_only();
    }
    void note_only()
    {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess && err == cudaSuccess)
            err = e;
    }
};

#define LP_LAUNCH(L, k, grid, block, ...) (L).launch(#k, k, grid, block, __VA_ARGS__)
#define LP_LAUNCH2D(L, k, grid, block, ...) (L).launch2d(#k, k, grid, block, __VA_ARGS__)
#define LP_LAUNCH_SMEM(L, k, grid, block, smem, ...) (L).launch_smem(#k, k, grid, block, smem, __VA_ARGS__)

// One-time kernel attributes (dynamic shared memory opt-in); called when a context is created.
void init_kernel_attributes();
void init_kdtree_attributes(); // lp_kdtree.cu
// Direct host I/O (lp_io.cu): inputs from and results into the caller's page-locked buffers.
void launch_io_in(Launcher& L, const BatchDev& b, const IoScan* io);
void launch_io_out(Launcher& L, const BatchDev& b, const IoScan* io, uint32_t* ret, int with_hull, int with_obb,
                   uint32_t nq);
void init_segment_tables(); // per-device constant tables (the seed-42 MT19937 stream)
// PointCloud2 bytes -> XYZI (+ ring) (lp_wire.cu); offsets: x, y, z, intensity, ring.
void launch_unpack_pointcloud2(cudaStream_t st, const uint8_t* data, uint32_t width, uint32_t height,
                               uint32_t point_step, uint32_t row_step, const uint32_t* offsets, float4* xyzi,
                               uint16_t* ring, uint64_t& launches);
// The processor's ground / obstacle / unsegmented clouds (lp_split.cu): out holds 3 x n records.
void launch_split_clouds(cudaStream_t st, const float4* pts, const uint32_t* labels, uint32_t n, lp_xyzrgb* out,
                         uint32_t* counts, uint32_t* sums, uint64_t& launches);
// Per-cluster products after the hulls (lp_objects.cu, k_obj_gate in lp_hull.cu).
struct RandWindow // glibc rand()'s last 34 values; pos: the slot the next value replaces
{
    uint32_t r[34];
    uint32_t pos;
};
struct VehicleTableDev // processor.hpp:60-192 in binary64: min/max length, width, height; bounds
{
    double dims[5][6];
    double bounds[5][4]; // min/max volume, min/max area
    double min_h, max_h, min_v, max_v;
};
struct ObjDev
{
    uint32_t K;
    const uint32_t* cl_off;   // K + 1: first cloud slot of each cluster
    const uint32_t* hull_off; // K + 1
    const int32_t* hull_idx;  // local indices
    const float* zmin;
    const float* zmax;
    int32_t* cls;             // K: vehicle type or -1
    lp_bounding_box* boxes;   // K: the gate's calipers boxes
    const lp_xyzrgb* cloud;   // the clustered cloud
    uint32_t* moff;           // K + 1: marker points per cluster -> exclusive scan
    double* mpts;             // marker points (3 doubles each)
    uint32_t mcap;
};
uint32_t obj_tiles(uint32_t n);
void launch_objects_cloud(cudaStream_t st, const float4* pts, const int32_t* labels, uint32_t n, uint32_t K,
                          uint32_t* cnt, uint32_t* sums, uint32_t* err, const RandWindow& w, uchar4* colour,
                          uint32_t* cl_off, lp_xyzrgb* cloud, uint64_t& launches);
void launch_objects_gates(cudaStream_t st, const ObjDev& o, const VehicleTableDev& vt, int enabled, double2* P,
                          float2* Pf, float* ea, int2* pairs, ScanState* state, uint64_t& launches);
void launch_objects_markers(cudaStream_t st, const ObjDev& o, uint32_t* sums, uint64_t& launches);

// Streaming multiprocessors of the current device (persistent grids are sized by it).
int sm_count();

// Host-side sizes of a batch (what the kernels' grids are sized by).
struct BatchHost
{
    int nscan = 0;
    bool any_compute_ring = false;
    bool any_noise = false;
    uint32_t ntiles = 0;
    uint32_t nslices = 0;
    std::vector<ScanDev> scans;
    // launch shapes (lp_tuning)
    uint32_t hull_ctas_per_sm = 2;
    uint32_t cell_ctas_per_sm = 8;
    uint32_t jcp_ctas_per_sm = 8;
};

void launch_segmentation(Launcher& L, const BatchDev& b, const BatchHost& hb, uint8_t* d_image);
void launch_ring_only(Launcher& L, const BatchDev& b, const BatchHost& hb);
void launch_clustering(Launcher& L, const BatchDev& b, const BatchHost& hb);
void launch_polygons(Launcher& L, const BatchDev& b, const BatchHost& hb, int compute_obb);
void launch_noise(Launcher& L, const BatchDev& b, const BatchHost& hb, const lp_noise_remover_config& cfg);
void launch_noise_compaction(Launcher& L, const BatchDev& b, const BatchHost& hb);
void launch_state_init(Launcher& L, const BatchDev& b, int noise);
void launch_outputs(Launcher& L, const BatchDev& b, int with_clusters);
void launch_mark_all_obstacles(Launcher& L, const BatchDev& b);
void launch_hull_single(Launcher& L, const double2* pts, uint32_t n, void* scratch, int* stack, int32_t* out,
                        uint32_t* n_out);
void launch_boxes_single(Launcher& L, const double2* P, uint32_t n, int2* pairs, int cap, int kind,
                         lp_bounding_box* out, int* npairs_out);
void launch_debug_math(Launcher& L, int kind, const float* a, const float* b, uint32_t n, float* out);
void launch_debug_math_sweep(Launcher& L, int kind, unsigned long long first, unsigned long long count,
                             unsigned long long* stats, unsigned long long* first_bad);
} // namespace lpg
