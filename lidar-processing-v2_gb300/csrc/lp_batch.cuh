// lp_batch.cuh — device pointers of one batch (passed by value to every kernel).
//
// HBM layout: each array is flat over the batch; scan s owns [ScanDev::*_off, + count).
//   points       float4 xyzi (16 B)            npts      (after optional noise compaction)
//   pixels       state u8, map i32, keys u64    npix      = sum H*W
//   polar cells  counts/starts/elevation        ncell     = sum nslice*nrad
//   near cells   RANSAC candidate counts        nnear     = sum nslice*4
//   obstacles    float4 + src index             <= npts
//   voxel hash   key/min/count                  nhash     = sum pow2 >= 2*n
//   clusters     counts/starts/boxes            ncl       = sum (n/min_size + 1)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lp_internal.cuh"

namespace lpg
{
// Pixel states of the range image (the reference's BGR colours, segmenter.hpp:144-148).
enum : uint8_t
{
    PX_EMPTY = 0,     // (0,0,0)
    PX_GROUND = 1,    // (0,255,0)
    PX_OBSTACLE = 2,  // (0,0,255)
    PX_INTERSECT = 4, // (255,0,0)   queued, not (yet) resolved by the vote
    PX_EMPTY_RED = 6, // (0,0,255)   empty pixel whose red channel was dilated
    PX_RES_G = 7,     // (0,255,0)   queued pixel the vote resolved to ground
    PX_RES_O = 8      // (0,0,255)   queued pixel the vote resolved to obstacle
};

// Vote outcomes / labels seen by a neighbour: 0 unknown, 1 ground, 2 obstacle.
enum : uint8_t
{
    V_U = 0,
    V_G = 1,
    V_O = 2
};

// Jump-convolution weight record of a queued pixel: 24 fresh weights, their sum, padding to a
// multiple of 16 bytes (vector loads).
constexpr uint32_t kKtPoolPerPoint = 8; // leftover search entries per point the DROR pool holds
constexpr uint32_t kJwStride = 28;
// Per image row of the jump convolution: lastq[3], pad, 24 stale weights, 24 stale label infos
// (kJrowNoUpdate: the row leaves the slot as it was; kJrowDynamic | pixel: the final colour of
// that pixel; else the label), padded to 64 words.
constexpr uint32_t kJrowWords = 64;
constexpr uint32_t kFinRingW = 4096; // image width up to which the vote keeps final colours in shared memory
// Staging of the vote's next row: queued pixels per row and image rows it covers, bytes per buffer
// (normalised records, the queue entries with 16-byte slack on both sides, the row record).
constexpr uint32_t kStageRec = 256;
constexpr uint32_t kRowCache = 1024;
constexpr uint32_t kStageRecBytes = kStageRec * kJwStride * 4u;
constexpr uint32_t kStageColBytes = (kStageRec * 2u + 32u + 15u) & ~15u;
constexpr uint32_t kStageBytes = kStageRecBytes + kStageColBytes + kJrowWords * 4u; // + the row record
constexpr uint32_t kJrowNoUpdate = 0xffffffffu;
constexpr uint32_t kJrowDynamic = 0x80000000u;

// A scan's buffers in the caller's page-locked host memory (device-accessible addresses).
struct IoScan
{
    const float* xyzi;
    const uint16_t* ring;
    uint8_t* noise;
    uint32_t* seg;
    int32_t* cl;
    uint32_t* hoff;
    int32_t* hidx;
    float* zmin;
    float* zmax;
    lp_bounding_box* obbc;
    lp_bounding_box* obbp;
    uint32_t cluster_cap, hull_cap;
    uint32_t q_off; // first 4-point chunk of the scan in the batch's chunk list
    uint32_t vec;   // 1: the label buffers allow 4-point vector stores (4 B noise, 16 B seg and cluster)
};

struct BatchDev
{
    int nscan;
    const ScanDev* scans;
    ScanState* state;

    // ---- input / points --------------------------------------------------------------------
    uint32_t nsrc;            // input points (before noise compaction)
    const float4* src;        // input points
    uint8_t* noise;           // per input point: LP_NOISE_*
    uint32_t* src_pos;        // per input point: compacted position (scan of VALID flags)
    uint32_t npts;            // points entering segmentation
    float4* pts;              // compacted points (== src when noise removal is off)
    int32_t* pt_src;          // compacted point -> input point (global)
    uint16_t* ring;           // per compacted point
    const uint16_t* ring_in;  // per input point, or null
    IoScan* io;               // per scan: the caller's page-locked buffers (direct host I/O)
    uint32_t* io_ret;         // per scan: hull index count written by the direct output kernel

    // ---- ring partition ---------------------------------------------------------------------
    uint8_t* quad;            // per point quadrant
    uint32_t ntiles;
    uint32_t* tile_cnt;       // transitions per 1024-point tile -> exclusive scan in place

    // ---- polar grid --------------------------------------------------------------------------
    int32_t* pt_cell;  // global cell or -1
    int32_t* pt_pix;   // local pixel h*W+w
    uint32_t* pt_slot; // arrival slot in the cell
    uint32_t ncell;
    uint32_t* cell_cnt;
    uint32_t* cell_start;
    int32_t* csr_idx;  // local point index per grid entry
    float* csr_z;
    float* zlow;       // per cell
    float* elev;       // per cell
    uint32_t* large_list;
    uint32_t* n_large;

    // ---- RANSAC ------------------------------------------------------------------------------
    uint32_t nnear;
    uint32_t* near_cnt;
    uint32_t* near_start;
    float4* cand;
    float4* planes;            // nscan * 60
    unsigned long long* pvalid; // nscan: bit it = hypothesis it usable
    uint32_t* inliers;         // nscan * 60

    // ---- projection / range image ------------------------------------------------------------
    uint8_t* pt_label; // per point after RECM + RANSAC
    uint32_t npix;
    uint32_t* pix_depth;
    unsigned long long* pix_key;
    int32_t* pix_map;
    uint8_t* pix_state;

    // ---- jump convolution -------------------------------------------------------------------
    uint32_t nrows;
    uint16_t* row_cols;        // per pixel slot: intersection columns of the row in order
    uint4* jq;            // flat list of the batch's queued pixels: (image row, position | column << 16, point, scan)
    uint32_t* row_cnt;         // per global row
    float* jw;                 // per row, its last three queued pixels: 24 fresh weights + sum (stride kJwStride)
    float* jn;                 // per queued pixel (flat queue position): 24 normalized weights, sum, slot label codes
    uint32_t* row_q0;          // per image row: its first position in the flat queue
    uint32_t jq_cap;           // queue capacity: sum over scans of min(pixels, points)
    uint32_t* jrow;            // per image row: kJrowWords words (lastq, stale-buffer update)
    unsigned long long* jmap;  // per entry: 9-state transition map

    // ---- segmentation output -----------------------------------------------------------------
    uint32_t* seg_label; // per compacted point

    // ---- clustering --------------------------------------------------------------------------
    uint32_t* obs_flag;   // per point: 1 if obstacle -> exclusive scan in place (obstacle slot)
    float4* obs_pts;      // per obstacle: x, y, z, (float)local index
    int32_t* obs_pt;      // per obstacle: compacted point index (global)
    float* obs_r;
    float* obs_a;
    float* obs_e;
    uint32_t* obs_hslot;  // per obstacle: hash slot
    uint32_t nhash;
    uint32_t* hkey;       // per slot: voxel flat key or 0xffffffff
    uint32_t* hmin;       // per slot: min local obstacle index
    uint32_t* hcnt;       // per slot: points in voxel
    uint32_t* hvid;       // per slot: number of occupied slots before it (voxel id of an occupied slot)
    uint32_t* vslot;      // per voxel id: hash slot
    uint32_t* parent;     // per voxel id
    uint32_t* cmin;       // per voxel id (valid at roots)
    uint32_t* ccnt;
    uint32_t* kflag;      // per obstacle: 1 at the min point of a kept component -> scan
    int32_t* obs_label;   // per obstacle: cluster label or -1

    // ---- per-cluster ---------------------------------------------------------------------------
    uint32_t ncl;
    uint32_t hull_cta_min; // clusters of more members take a CTA of the hull kernel (tuning)
    uint32_t* cl_cnt;     // members per cluster
    uint32_t* cl_start;   // exclusive scan of cl_cnt
    uint32_t* cl_fill;
    uint32_t* members;    // obstacle indices grouped by cluster (unordered within)
    float2* mxy;          // x, y of each member, by member slot
    uint32_t* cl_zkey;    // per cluster: max of ~ord(z) (the lowest z), max of ord(z) (the highest)
    uint32_t* hull_cnt;   // hull vertices per cluster -> exclusive scan in place
    int32_t* hull_tmp;    // per member slot: hull local indices at cl_start
    int32_t* hull_out;    // dense hull local indices (batch)
    float* cl_zmin;
    float* cl_zmax;
    lp_bounding_box* obb_c;
    lp_bounding_box* obb_p;
    void* hs_cand;        // hull candidates (12 B each), 2 per member slot, at 2 * cl_start
    int32_t* hs_stack;    // monotone-chain stack, at 2 * cl_start + 2 * cluster
    double2* hs_pts;      // hull vertices as FP64, at cl_start
    int2* hs_pairs;       // antipodal pairs, at 4 * cl_start + 16 * cluster
    uint32_t* queue;      // [0] clusters in the batch, [1] hull work-queue head, [4] tie clusters
    uint32_t* tie_list;
    uint2* pre_items;          // (cluster, chunk) items of the large clusters' member passes
    unsigned long long* pre_ext;  // per cluster: its 16 direction extremes (packed keys)
    unsigned long long* pre_pk;   // per cluster: the farthest member outside each edge of the first polygon
    uint32_t* pre_nact;        // per cluster: members not inside the first polygon (listed in the chain scratch)   // clusters whose hull has a vertex with an identical point (reference tie order)

    // ---- DROR (reference kd-tree replay, lp_kdtree.cu) ------------------------------------------
    float4* kt;                // per input point: tree node record by position (x, y, z, subtree size bits)
    float4* kbb;               // 2 per input point: subtree box (lo, hi) by node position
    uint32_t* kscr;            // 2 per input point: candidate positions of the parallel partition (later,
                               // per candidate: its walk through its predecessor's stop pieces: stop entry, left at)
    uint32_t* kown;            // per point: count of its own search (capped at min_neighbours); later, per
                               // candidate: the count after that walk
    uint32_t* kshort;          // per point (+1): 1 if its own search fell short -> exclusive scan
    uint32_t* klo_n;           // per point (+1): entries its search left behind; later, per short point:
                               // the first flat entry of its piece
    uint32_t* klo_off;         // exclusive scan of klo_n: their place in kflat
    uint32_t* klo_at;          // per point: their place in kpool; later, per candidate: that walk's status,
                               // left count and stop piece
    uint32_t* kpool;           // leftover entries as searches produce them (kpool_cap)
    uint32_t* kflat;           // the points' leftovers in point order (kpool_cap)
    uint32_t kpool_cap;
    uint32_t* kq;              // short points in order (before that, from the build to the own search:
                               // the input index of the point at each tree position)
    uint4* kc;                 // per short point: count, stop entry, left entries (pool at, count)
    uint32_t* kcflag;          // per short point (+1): 1 if step 3 left it undecided -> exclusive scan
    uint32_t* kcand;           // those candidates (short indices) in order
    uint4* kspec;              // per candidate: count, stop short index, stop entry | kind << 31, left at
    uint32_t* kspec_n;         // per candidate: entries the stopping search left
    uint2* kpiece;             // per scan: stack of pieces (2 n + 2 per scan)
    uint32_t* kctr;            // [0] pool head

    // ---- outputs per input point ---------------------------------------------------------------
    uint32_t* out_seg;
    int32_t* out_cl;
};

__device__ __forceinline__ int scan_of_point(const BatchDev& b, uint32_t i)
{
    return find_scan(b.nscan, i, [&](int s) { return b.scans[s].pt_off; });
}
} // namespace lpg
