// lp_runtime.hpp — host runtime shared by the C ABI (lp_api.cu) and the serving loop
// (lp_serve.cu): contexts, batches and the plan/upload/execute/download steps of a batch.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "lidar_gb300.h"
#include "lidar_gb300_batch.h"
#include "lp_batch.cuh"
#include "lp_stages.hpp"

namespace lprt
{
enum Stage : uint32_t
{
    ST_RING = 1u << 0,    // ring partition (lp_add_ring_info)
    ST_NOISE = 1u << 1,   // DROR on the input cloud
    ST_SEG = 1u << 2,     // segmentation
    ST_CLUSTER = 1u << 3, // cluster the obstacle points
    ST_HULL = 1u << 4,
    ST_OBB = 1u << 5,
    ST_ALL_OBS = 1u << 6, // cluster the whole input (lp_cluster)
    ST_IMAGE = 1u << 7,
};

struct ScanIn
{
    const float* xyzi = nullptr; // host
    uint32_t stride = 4;         // floats between points
    const uint16_t* ring = nullptr;
    uint32_t n = 0;
    lp_segmenter_config seg{};
    int32_t compute_ring = 0;
    int32_t first_ring = 0;
};

lp_tuning tuning_default(); // lp_tune.cu

struct Run
{
    uint32_t stages = 0;
    lp_clusterer_config cl{};
    lp_noise_remover_config nr{};
    std::vector<ScanIn> scans;
};
} // namespace lprt

struct lp_context
{
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t launches = 0;
    std::string last_error;
    std::vector<cudaEvent_t> events;
    lp_batch* cached = nullptr;
    // lp_process_batch on page-locked buffers with 16 or more scans: concurrent parts, each with
    // its own stream and device region, reused call after call
    std::vector<lp_batch*> cached_parts;
    cudaEvent_t fork = nullptr;
    void* split_mem = nullptr; // lp_split_clouds scratch
    size_t split_cap = 0;
    void* flush = nullptr; // buffer larger than L2 for cache flushing between timed runs
    size_t flush_bytes = 0;
    // lp_cluster_objects: glibc rand() positioned at the last call's first draw (advanced, not
    // recomputed, when the next call's offset lies ahead)
    uint64_t rand_at = 0;
    bool rand_valid = false;
    lpg::RandWindow rand_window{};
    // lp_context_set_tuning_table: bucket (lprt::key_index) -> tuning for batches created here
    std::map<uint32_t, lp_tuning> tuning;
};

struct lp_batch
{
    lprt::Run run;
    lpg::BatchHost hb;
    lpg::BatchDev b{};
    char* mem = nullptr;
    size_t cap = 0;
    uint32_t* scan_sums = nullptr;
    uint8_t* d_image = nullptr;
    std::vector<lpg::ScanState> h_state;
    std::vector<float4> staging; // host repack for stride-3 inputs
    cudaGraphExec_t graph = nullptr;
    std::vector<lpg::LaunchRecord> prof;
    bool profiling = false;
    // A part of a split batch runs on its own stream (null: the context stream).
    cudaStream_t stream = nullptr;
    // A split batch: scan i lives in parts[i % parts.size()] at position i / parts.size(); the parts
    // run concurrently on their streams (fork from and join into the context stream), so one
    // part's latency-bound tails overlap the others' work.
    std::vector<lp_batch*> parts;
    std::vector<std::vector<uint32_t>> part_scans; // the batch's scan indices in part k, in batch order
    std::vector<cudaEvent_t> fork_join;            // [0] fork, [1 + k] part k done
    lp_tuning tune = lprt::tuning_default();       // the batch's split and launch shapes
    std::vector<uint32_t> h_nh;         // direct host I/O: hull index count per scan (read back)
};

namespace lprt
{
lp_status fail(lp_context* ctx, lp_status st, const std::string& msg);
// Layout of the batch on the host (no device work).
lp_status plan(lp_context* ctx, lp_batch& B);
// Device bytes a planned batch needs (carve with a null base).
size_t measure(lp_batch& B);
// plan + (re)allocate + carve.
lp_status build(lp_context* ctx, lp_batch& B);
lp_status upload(lp_context* ctx, lp_batch& B);
lp_status execute(lp_context* ctx, lp_batch& B);
lp_status fetch_state(lp_context* ctx, lp_batch& B);
lp_status download(lp_context* ctx, lp_batch& B, lp_scan_output* outs);
lp_status fill_pipeline(lp_context* ctx, lp_batch& B, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                        uint32_t nscans);
void destroy_batch(lp_batch* B);
// Tuning (lp_tune.cu): bucket index of a key, the tuning a batch of these scans takes in this
// context, the number of parts and which scans go to each.
uint32_t key_index(const lp_tuning_key& k);
lp_tuning_key key_of(const lp_scan_input* scans, uint32_t nscans);
lp_tuning tuning_for(const lp_context* ctx, const lp_scan_input* scans, uint32_t nscans);
uint32_t part_count(const lp_tuning& t, uint32_t nscans);
std::vector<std::vector<uint32_t>> assign_parts(const lp_scan_input* scans, uint32_t nscans, uint32_t parts,
                                                bool balance);
} // namespace lprt
