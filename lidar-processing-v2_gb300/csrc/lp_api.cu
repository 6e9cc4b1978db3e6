// lp_api.cu — context, batch planning/allocation and the C ABI of liblp_gpu.so.
//
// A context is one CUDA stream. A batch owns one device allocation holding every array of the
// launch sequence (inputs stay resident, so a prepared batch can be re-executed or captured as
// a CUDA graph). A batch of 16 or more scans is split into up to eight parts, each its own batch on
// its own stream, forked from and joined into the context stream. A one-shot call (lp_segment,
// lp_process_batch, ...) reuses batches cached in the context: plan on the host, upload, run the
// whole sequence without host syncs, read the small per-scan state, then the results. All waits
// inside kernels are bounded.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "lidar_gb300.h"
#include "lidar_gb300_batch.h"
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_runtime.hpp"
#include "lp_stages.hpp"

using namespace lpg;

namespace
{
constexpr float kDegToRad = static_cast<float>(M_PI / 180.0); // segmenter.hpp:135, clusterer.hpp:78
constexpr float kTwoPiF = static_cast<float>(2.0 * M_PI);     // segmenter.hpp:136
} // namespace

namespace lprt
{
lp_status fail(lp_context* ctx, lp_status st, const std::string& msg)
{
    if (ctx)
        ctx->last_error = msg;
    return st;
}

lp_status cuda_fail(lp_context* ctx, cudaError_t e, const char* where)
{
    cudaGetLastError();
    return fail(ctx, LP_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define LP_CUDA(ctx, call)                                                                                  \
    do                                                                                                      \
    {                                                                                                       \
        const cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess)                                                                              \
            return cuda_fail(ctx, e_, #call);                                                               \
    } while (0)

#define LP_TRY(call)                                                                                        \
    do                                                                                                      \
    {                                                                                                       \
        const lp_status s_ = (call);                                                                        \
        if (s_ != LP_OK)                                                                                    \
            return s_;                                                                                      \
    } while (0)

struct Carver
{
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(size_t count)
    {
        off = (off + 255) & ~static_cast<size_t>(255);
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += count * sizeof(T) + 16;
        return p;
    }
};

bool seg_config_ok(const lp_segmenter_config& c)
{
    if (c.image_width <= 0 || c.image_height <= 0 || c.image_width > 65535 || c.image_height > 65535)
        return false;
    if (!(c.grid_radial_spacing_m > 0) || !(c.grid_slice_resolution_deg > 0) || !(c.max_distance_m > 0))
        return false;
    const float slice_res = c.grid_slice_resolution_deg * kDegToRad;
    const int32_t nrad = static_cast<int32_t>(c.max_distance_m / c.grid_radial_spacing_m);
    const int32_t nslice = static_cast<int32_t>(kTwoPiF / slice_res);
    return nrad >= kRansacRadialBins && nslice >= 1 && static_cast<int64_t>(nrad) * nslice < (1 << 24) &&
           static_cast<int64_t>(c.image_width) * c.image_height < (1 << 28);
}

// Host-side layout and the configuration constants of every scan (binary32 expressions
// evaluated exactly as the reference writes them).
lp_status plan(lp_context* ctx, lp_batch& B)
{
    const Run& R = B.run;
    BatchHost& hb = B.hb;
    hb = BatchHost{};
    hb.nscan = static_cast<int>(R.scans.size());
    hb.any_noise = (R.stages & ST_NOISE) != 0;
    uint64_t pt = 0, pix = 0, row = 0, tile = 0, slice = 0, cell = 0, nearc = 0, hash = 0, cl = 0, queue = 0;
    const bool seg = (R.stages & ST_SEG) != 0;
    for (const ScanIn& in : R.scans)
    {
        ScanDev sd{};
        sd.pt_off = static_cast<uint32_t>(pt);
        sd.n = in.n;
        sd.src_off = static_cast<uint32_t>(pt);
        sd.n_src = in.n;
        sd.tile_off = static_cast<uint32_t>(tile);
        sd.compute_ring = in.compute_ring;
        if (in.compute_ring)
            hb.any_compute_ring = true;
        sd.first_ring = in.first_ring;
        if (seg)
        {
            const lp_segmenter_config& c = in.seg;
            if (!seg_config_ok(c))
                return fail(ctx, LP_ERR_BAD_ARG, "segmenter configuration out of the supported range");
            sd.H = c.image_height;
            sd.W = c.image_width;
            sd.pix_off = static_cast<uint32_t>(pix);
            sd.row_off = static_cast<uint32_t>(row);
            sd.slice_res = c.grid_slice_resolution_deg * kDegToRad; // segmenter.cpp:42-46
            sd.nrad = static_cast<int32_t>(c.max_distance_m / c.grid_radial_spacing_m);
            sd.nslice = static_cast<int32_t>(kTwoPiF / sd.slice_res);
            sd.cell_off = static_cast<uint32_t>(cell);
            sd.slice_off = static_cast<uint32_t>(slice);
            sd.nnear_per_slice = std::min(kRansacRadialBins, sd.nrad);
            sd.near_off = static_cast<uint32_t>(nearc);
            const float up = c.elevation_up_deg * kDegToRad; // segmenter.cpp:106-109
            const float down = c.elevation_down_deg * kDegToRad;
            const float vfov = up - down;
            sd.rad_per_px = vfov / static_cast<float>(c.image_height);
            sd.down_rad = down;
            sd.zmin_adj = -c.sensor_height_m + c.z_min_m; // segmenter.cpp:121-122
            sd.zmax_adj = -c.sensor_height_m + c.z_max_m;
            sd.spacing = c.grid_radial_spacing_m;
            sd.min_d = c.min_distance_m;
            sd.max_d = c.max_distance_m;
            sd.delta = std::min(c.grid_radial_spacing_m * std::tan(c.road_maximum_slope_m_per_m), // :209-211
                                c.ground_height_threshold_m - std::numeric_limits<float>::epsilon());
            sd.thr = c.ground_height_threshold_m;
            sd.sensor_h = c.sensor_height_m;
            sd.kthr2 = c.kernel_threshold_distance_m * c.kernel_threshold_distance_m; // :532-533
            sd.amp = c.amplification_factor;
            sd.max_cos = std::cos(std::tan(c.road_maximum_slope_m_per_m)); // :360
            sd.use_ring = ((in.ring != nullptr) || in.compute_ring) && !c.assume_unorganized_cloud;
            if (sd.compute_ring && sd.first_ring < 0)
                sd.first_ring = c.image_height - 1;
            pix += static_cast<uint64_t>(sd.H) * static_cast<uint64_t>(sd.W);
            // a queued pixel of the vote holds a point: at most min(pixels, points) per scan
            queue += std::min<uint64_t>(static_cast<uint64_t>(sd.H) * static_cast<uint64_t>(sd.W), in.n);
            row += static_cast<uint64_t>(sd.H);
            cell += static_cast<uint64_t>(sd.nslice) * static_cast<uint64_t>(sd.nrad);
            slice += static_cast<uint64_t>(sd.nslice);
            nearc += static_cast<uint64_t>(sd.nslice) * static_cast<uint64_t>(sd.nnear_per_slice);
        }
        else if (sd.compute_ring && sd.first_ring < 0)
        {
            sd.first_ring = 63; // dataloader.cpp:87
        }
        sd.res_r = R.cl.voxel_grid_range_resolution_m; // Clusterer::config, clusterer.hpp:76-84
        sd.res_a = R.cl.voxel_grid_azimuth_resolution_deg * kDegToRad;
        sd.res_e = R.cl.voxel_grid_elevation_resolution_deg * kDegToRad;
        sd.min_cluster = R.cl.min_cluster_size;
        sd.hash_off = static_cast<uint32_t>(hash);
        sd.hash_cap = next_pow2(std::max(64u, 2u * in.n));
        const uint32_t minc = std::max(1u, R.cl.min_cluster_size);
        sd.cluster_cap = in.n / minc + 1;
        sd.cl_off = static_cast<uint32_t>(cl);
        sd.hull_cap = in.n;
        sd.dror_s2 = std::pow(static_cast<double>(R.nr.radius_multiplier_m_per_m), 2.0); // noise_remover.cpp:49-52
        sd.dror_rmin2 = R.nr.min_search_radius_m * R.nr.min_search_radius_m;
        sd.dror_k = R.nr.min_neighbours;
        pt += in.n;
        tile += div_up(std::max(in.n, 1u), 1024u);
        hash += sd.hash_cap;
        cl += sd.cluster_cap;
        hb.scans.push_back(sd);
    }
    const uint64_t lim = 0x7fffffffull;
    if (pt > lim / 8 || pix > lim / 8 || hash > lim || cell > lim || cl > lim)
        return fail(ctx, LP_ERR_CAPACITY, "batch too large for 32-bit indexing; split it");
    hb.ntiles = static_cast<uint32_t>(tile);
    hb.nslices = static_cast<uint32_t>(slice);
    hb.hull_ctas_per_sm = B.tune.hull_ctas_per_sm;
    hb.cell_ctas_per_sm = B.tune.cell_ctas_per_sm;
    hb.jcp_ctas_per_sm = B.tune.jcp_ctas_per_sm;
    BatchDev& b = B.b;
    b = BatchDev{};
    b.nscan = hb.nscan;
    b.hull_cta_min = B.tune.hull_cta_min;
    b.nsrc = static_cast<uint32_t>(pt);
    b.npts = static_cast<uint32_t>(pt);
    b.ntiles = static_cast<uint32_t>(tile);
    b.ncell = static_cast<uint32_t>(cell);
    b.nnear = static_cast<uint32_t>(nearc);
    b.npix = static_cast<uint32_t>(pix);
    b.nrows = static_cast<uint32_t>(row);
    b.nhash = static_cast<uint32_t>(hash);
    b.ncl = static_cast<uint32_t>(cl);
    b.jq_cap = static_cast<uint32_t>(queue);
    return LP_OK;
}

// Lays out every array of the batch (pass 1 with base == nullptr measures the size).
size_t carve(lp_batch& B, char* base)
{
    BatchDev& b = B.b;
    const Run& R = B.run;
    const uint32_t N = b.npts, S = static_cast<uint32_t>(b.nscan);
    const bool seg = R.stages & ST_SEG;
    const bool clu = R.stages & (ST_CLUSTER | ST_ALL_OBS);
    const bool hull = R.stages & ST_HULL;
    const bool noise = R.stages & ST_NOISE;
    const bool ring_in = std::any_of(R.scans.begin(), R.scans.end(), [](const ScanIn& s) { return s.ring != nullptr; });
    Carver c{base};
    auto put = [&](auto*& field, size_t count) {
        using T = std::remove_reference_t<decltype(*field)>;
        field = c.take<std::remove_const_t<T>>(count);
    };
    ScanDev* scans;
    put(scans, S);
    b.scans = scans;
    put(b.state, S);
    put(b.io, S);
    put(b.io_ret, S);
    const uint32_t maxlen = std::max({N, b.npix, b.nhash, b.ncell, b.ncl, b.ntiles, b.nnear}) + 2;
    put(B.scan_sums, div_up(maxlen, static_cast<uint32_t>(kScanTile)) + 4);
    float4* src;
    put(src, N);
    b.src = src;
    b.ring_in = nullptr;
    if (ring_in)
    {
        uint16_t* r;
        put(r, N);
        b.ring_in = r;
    }
    put(b.noise, N);
    put(b.ring, N);
    if (noise)
    {
        put(b.src_pos, N + 1);
        put(b.pts, N);
        put(b.pt_src, N);
        // kd-tree replay (lp_kdtree.cu): leftover pool of kKtPoolPerPoint entries per point (the
        // searches leave about 4 per point; a fuller pool is reported as a capacity error)
        b.kpool_cap = static_cast<uint32_t>(std::min<uint64_t>(static_cast<uint64_t>(kKtPoolPerPoint) * N + 64, 0x7fffffffull));
        put(b.kt, N);
        put(b.kbb, 2ull * N);
        put(b.kscr, 2ull * N);
        put(b.kown, N);
        put(b.kshort, N + 1);
        put(b.klo_n, N + 1);
        put(b.klo_off, N + 1);
        put(b.klo_at, N);
        put(b.kpool, b.kpool_cap);
        put(b.kflat, b.kpool_cap);
        put(b.kq, N);
        put(b.kc, N);
        put(b.kcflag, N + 1);
        put(b.kcand, N);
        put(b.kspec, N);
        put(b.kspec_n, N);
        put(b.kpiece, 2ull * N + 2ull * S);
        put(b.kctr, 4);
    }
    else
    {
        b.pts = src;
        b.pt_src = nullptr;
    }
    put(b.quad, N);
    put(b.tile_cnt, b.ntiles + 1);
    put(b.seg_label, N);
    put(b.out_seg, N);
    put(b.out_cl, N);
    B.d_image = nullptr;
    if (seg)
    {
        put(b.pt_cell, N);
        put(b.pt_pix, N);
        put(b.pt_slot, N);
        put(b.cell_cnt, b.ncell + 1);
        put(b.cell_start, b.ncell + 1);
        put(b.csr_idx, N);
        put(b.csr_z, N);
        put(b.zlow, b.ncell);
        put(b.elev, b.ncell);
        put(b.large_list, b.ncell);
        put(b.n_large, 1);
        put(b.near_cnt, b.nnear + 1);
        put(b.near_start, b.nnear + 1);
        put(b.cand, N);
        put(b.planes, S * kMaxRansacIters);
        put(b.pvalid, S);
        put(b.inliers, S * kMaxRansacIters);
        put(b.pt_label, N);
        put(b.pix_depth, b.npix);
        put(b.pix_key, b.npix);
        put(b.pix_map, b.npix);
        put(b.pix_state, b.npix);
        put(b.row_cols, b.npix);
        put(b.row_cnt, b.nrows + 1); // [nrows]: queued pixels of the batch
        put(b.row_q0, b.nrows);
        put(b.jq, b.jq_cap + 1);
        put(b.jw, static_cast<size_t>(b.nrows) * 3u * kJwStride); // the last three queued pixels of each row
        put(b.jn, (static_cast<size_t>(b.jq_cap) + 1) * kJwStride);
        put(b.jrow, static_cast<size_t>(b.nrows) * kJrowWords);
        put(b.jmap, b.jq_cap + 1);
        if (R.stages & ST_IMAGE)
            put(B.d_image, static_cast<size_t>(b.npix) * 3);
    }
    if (clu)
    {
        put(b.obs_flag, N + 1);
        put(b.obs_pts, N);
        put(b.obs_pt, N);
        put(b.obs_r, N);
        put(b.obs_a, N);
        put(b.obs_e, N);
        put(b.obs_hslot, N);
        put(b.hkey, b.nhash);
        put(b.hmin, b.nhash);
        put(b.hcnt, b.nhash);
        put(b.hvid, b.nhash + 1);
        put(b.vslot, b.nhash);
        put(b.parent, b.nhash);
        put(b.cmin, b.nhash);
        put(b.ccnt, b.nhash);
        put(b.kflag, N + 1);
        put(b.obs_label, N);
        put(b.cl_cnt, b.ncl + 1);
        put(b.cl_start, b.ncl + 1);
        put(b.cl_fill, b.ncl + 1);
        put(b.members, N);
        put(b.mxy, N);
        put(b.cl_zkey, 2ull * b.ncl);
    }
    if (hull)
    {
        put(b.hull_cnt, b.ncl + 1);
        put(b.hull_tmp, N);
        put(b.hull_out, N);
        put(b.cl_zmin, b.ncl);
        put(b.cl_zmax, b.ncl);
        put(b.obb_c, b.ncl);
        put(b.obb_p, b.ncl);
        uint8_t* cand;
        put(cand, static_cast<size_t>(2) * N * 12 + 64);
        b.hs_cand = cand;
        put(b.hs_stack, static_cast<size_t>(2) * N + 2ull * b.ncl + 8);
        put(b.hs_pts, static_cast<size_t>(N) + 8);
        put(b.hs_pairs, static_cast<size_t>(4) * N + 16ull * b.ncl + 16);
        put(b.queue, 8);
        put(b.tie_list, b.ncl + 1);
        put(b.pre_items, N / 4096u + b.ncl + 1);
        put(b.pre_ext, 16ull * b.ncl + 16);
        put(b.pre_pk, 16ull * b.ncl + 16);
        put(b.pre_nact, b.ncl + 1);
    }
    return c.off + 4096;
}

lp_status build(lp_context* ctx, lp_batch& B)
{
    LP_TRY(plan(ctx, B));
    const size_t bytes = carve(B, nullptr);
    if (bytes > B.cap)
    {
        if (B.graph)
        {
            cudaGraphExecDestroy(B.graph);
            B.graph = nullptr;
        }
        if (B.mem)
        {
            cudaStreamSynchronize(ctx->stream);
            if (B.stream)
                cudaStreamSynchronize(B.stream);
            cudaFree(B.mem);
            B.mem = nullptr;
            B.cap = 0;
        }
        const size_t cap = bytes + bytes / 8;
        LP_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&B.mem), cap));
        B.cap = cap;
    }
    carve(B, B.mem);
    B.h_state.assign(B.hb.nscan, ScanState{});
    return LP_OK;
}

lp_status upload(lp_context* ctx, lp_batch& B)
{
    BatchDev& b = B.b;
    const cudaStream_t st = ctx->stream;
    LP_CUDA(ctx, cudaMemcpyAsync(const_cast<ScanDev*>(b.scans), B.hb.scans.data(),
                                 B.hb.scans.size() * sizeof(ScanDev), cudaMemcpyHostToDevice, st));
    for (size_t s = 0; s < B.run.scans.size(); ++s)
    {
        const ScanIn& in = B.run.scans[s];
        const ScanDev& sd = B.hb.scans[s];
        if (in.n == 0)
            continue;
        float4* dst = const_cast<float4*>(b.src) + sd.src_off;
        if (in.stride == 4)
        {
            LP_CUDA(ctx, cudaMemcpyAsync(dst, in.xyzi, static_cast<size_t>(in.n) * 16, cudaMemcpyHostToDevice, st));
        }
        else
        {
            B.staging.resize(in.n);
            for (uint32_t i = 0; i < in.n; ++i)
                B.staging[i] = make_float4(in.xyzi[static_cast<size_t>(in.stride) * i],
                                           in.xyzi[static_cast<size_t>(in.stride) * i + 1],
                                           in.xyzi[static_cast<size_t>(in.stride) * i + 2], 0.0f);
            LP_CUDA(ctx, cudaMemcpyAsync(dst, B.staging.data(), static_cast<size_t>(in.n) * 16, cudaMemcpyHostToDevice, st));
            LP_CUDA(ctx, cudaStreamSynchronize(st)); // staging is reused by the next scan
        }
        if (in.ring && b.ring_in)
            LP_CUDA(ctx, cudaMemcpyAsync(const_cast<uint16_t*>(b.ring_in) + sd.src_off, in.ring,
                                         static_cast<size_t>(in.n) * 2, cudaMemcpyHostToDevice, st));
    }
    return LP_OK;
}

// The whole launch sequence of a batch (memsets + kernels), no host synchronisation.
lp_status execute(lp_context* ctx, lp_batch& B)
{
    BatchDev& b = B.b;
    const Run& R = B.run;
    const cudaStream_t st = B.stream ? B.stream : ctx->stream;
    Launcher L;
    L.stream = st;
    L.launches = &ctx->launches;
    L.scan_sums = B.scan_sums;
    L.scan_err = &b.state->err; // scan 0's error word: a failed scan fails the batch
    L.event_pool = &ctx->events;
    if (B.profiling)
        L.prof = &B.prof;
    const uint32_t N = b.npts, S = static_cast<uint32_t>(b.nscan);
    LP_CUDA(ctx, cudaMemsetAsync(b.state, 0, S * sizeof(ScanState), st));
    LP_CUDA(ctx, cudaMemsetAsync(b.seg_label, 0, static_cast<size_t>(N) * 4, st));
    LP_CUDA(ctx, cudaMemsetAsync(b.out_seg, 0, static_cast<size_t>(N) * 4, st));
    LP_CUDA(ctx, cudaMemsetAsync(b.out_cl, 0xff, static_cast<size_t>(N) * 4, st));
    const bool noise = R.stages & ST_NOISE;
    if (!noise)
        LP_CUDA(ctx, cudaMemsetAsync(b.noise, 0, N, st));
    if (b.ring_in && !noise)
        LP_CUDA(ctx, cudaMemcpyAsync(b.ring, b.ring_in, static_cast<size_t>(N) * 2, cudaMemcpyDeviceToDevice, st));
    launch_state_init(L, b, noise ? 1 : 0);
    if (noise)
    {
        launch_noise(L, b, B.hb, R.nr);
        if (R.stages & (ST_SEG | ST_CLUSTER | ST_ALL_OBS | ST_RING))
            launch_noise_compaction(L, b, B.hb);
    }
    if (R.stages & (ST_RING | ST_SEG))
    {
        LP_CUDA(ctx, cudaMemsetAsync(b.tile_cnt, 0, (static_cast<size_t>(b.ntiles) + 1) * 4, st));
    }
    if ((R.stages & ST_RING) && !(R.stages & ST_SEG))
        launch_ring_only(L, b, B.hb);
    if (R.stages & ST_SEG)
    {
        LP_CUDA(ctx, cudaMemsetAsync(b.cell_cnt, 0, (static_cast<size_t>(b.ncell) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.n_large, 0, 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.near_cnt, 0, (static_cast<size_t>(b.nnear) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.pix_depth, 0xff, static_cast<size_t>(b.npix) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.pix_key, 0xff, static_cast<size_t>(b.npix) * 8, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.row_cnt, 0, (static_cast<size_t>(b.nrows) + 1) * 4, st));
        launch_segmentation(L, b, B.hb, B.d_image);
    }
    if (R.stages & ST_ALL_OBS)
        launch_mark_all_obstacles(L, b);
    if (R.stages & (ST_CLUSTER | ST_ALL_OBS))
    {
        LP_CUDA(ctx, cudaMemsetAsync(b.hkey, 0xff, static_cast<size_t>(b.nhash) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.hmin, 0xff, static_cast<size_t>(b.nhash) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.hcnt, 0, static_cast<size_t>(b.nhash) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.kflag, 0, (static_cast<size_t>(N) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.cl_cnt, 0, (static_cast<size_t>(b.ncl) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.cl_fill, 0, (static_cast<size_t>(b.ncl) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.cl_zkey, 0, static_cast<size_t>(b.ncl) * 8, st));
        launch_clustering(L, b, B.hb);
    }
    if (R.stages & ST_HULL)
    {
        LP_CUDA(ctx, cudaMemsetAsync(b.hull_cnt, 0, (static_cast<size_t>(b.ncl) + 1) * 4, st));
        LP_CUDA(ctx, cudaMemsetAsync(b.queue, 0, 8 * 4, st));
        launch_polygons(L, b, B.hb, (R.stages & ST_OBB) ? 1 : 0);
    }
    if (R.stages & (ST_SEG | ST_CLUSTER | ST_ALL_OBS))
        launch_outputs(L, b, (R.stages & (ST_CLUSTER | ST_ALL_OBS)) ? 1 : 0);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "kernel launch");
    return LP_OK;
}

lp_status report_state(lp_context* ctx, lp_batch& B);

lp_status fetch_state(lp_context* ctx, lp_batch& B)
{
    LP_CUDA(ctx, cudaMemcpyAsync(B.h_state.data(), B.b.state, B.h_state.size() * sizeof(ScanState),
                                 cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return report_state(ctx, B);
}

// Status of a batch from the fetched per-scan error words.
lp_status report_state(lp_context* ctx, lp_batch& B)
{
    lp_status worst = LP_OK;
    for (size_t s = 0; s < B.h_state.size(); ++s)
    {
        const uint32_t e = B.h_state[s].err;
        if (!e)
            continue;
        lp_status st = LP_ERR_INTERNAL;
        std::string what;
        if (e & (ERR_VOXEL_CAPACITY | ERR_CLUSTER_CAPACITY | ERR_CELL_TOO_LARGE | ERR_HASH_FULL | ERR_HULL_CAPACITY))
        {
            st = LP_ERR_CAPACITY;
            what = (e & ERR_VOXEL_CAPACITY) ? "more than 200000 occupied voxels (Exceeded reserved element capacity)"
                                            : "a fixed capacity was exceeded";
        }
        else if (e & ERR_UF_TIMEOUT)
        {
            st = LP_ERR_TIMEOUT;
            what = "union-find iteration limit reached";
        }
        else
        {
            what = "device consistency check failed";
        }
        ctx->last_error = "scan " + std::to_string(s) + ": " + what;
        if (worst == LP_OK)
            worst = st;
    }
    return worst;
}

lp_status ensure_device(lp_context* ctx)
{
    LP_CUDA(ctx, cudaSetDevice(ctx->device));
    return LP_OK;
}

lp_batch& cached(lp_context* ctx)
{
    if (!ctx->cached)
        ctx->cached = new lp_batch();
    return *ctx->cached;
}

void destroy_batch(lp_batch* B)
{
    if (!B)
        return;
    if (B->graph)
        cudaGraphExecDestroy(B->graph);
    if (B->mem)
        cudaFree(B->mem);
    for (lp_batch* P : B->parts)
        destroy_batch(P);
    for (cudaEvent_t e : B->fork_join)
        cudaEventDestroy(e);
    if (B->stream)
        cudaStreamDestroy(B->stream);
    delete B;
}

// Launches a batch: a split batch forks its parts' streams from the context stream, launches every
// part on its own stream and joins them back (also the shape a graph capture records).
lp_status launch_batch(lp_context* ctx, lp_batch& B)
{
    if (B.parts.empty())
        return execute(ctx, B);
    LP_CUDA(ctx, cudaEventRecord(B.fork_join[0], ctx->stream));
    for (size_t k = 0; k < B.parts.size(); ++k)
    {
        lp_batch& P = *B.parts[k];
        LP_CUDA(ctx, cudaStreamWaitEvent(P.stream, B.fork_join[0], 0));
        LP_TRY(execute(ctx, P));
        LP_CUDA(ctx, cudaEventRecord(B.fork_join[1 + k], P.stream));
    }
    for (size_t k = 0; k < B.parts.size(); ++k)
        LP_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, B.fork_join[1 + k], 0));
    return LP_OK;
}

lp_status run_once(lp_context* ctx, lp_batch& B)
{
    LP_TRY(build(ctx, B));
    LP_TRY(upload(ctx, B));
    LP_TRY(execute(ctx, B));
    return fetch_state(ctx, B);
}

lp_status copy_d2h(lp_context* ctx, void* dst, const void* src, size_t bytes)
{
    if (!dst || bytes == 0)
        return LP_OK;
    LP_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return LP_OK;
}

// Per-scan results of a pipeline batch into the caller's lp_scan_output structs. Two phases with
// one stream synchronisation each: first the labels and every scan's hull-offset range (cluster
// counts are known from the fetched state), then, with the offsets on the host, the hull indices,
// z ranges and boxes. Copies into page-locked caller buffers run asynchronously.
lp_status download(lp_context* ctx, lp_batch& B, lp_scan_output* outs)
{
    const BatchDev& b = B.b;
    const bool hull = B.run.stages & ST_HULL;
    const size_t S = B.run.scans.size();
    std::vector<size_t> hbase(S + 1, 0);
    for (size_t s = 0; s < S; ++s)
        hbase[s + 1] = hbase[s] + (hull ? static_cast<size_t>(B.h_state[s].n_clusters) + 1 : 0);
    std::vector<uint32_t> hoff(hbase[S]);
    for (size_t s = 0; s < S; ++s)
    {
        const ScanDev& sd = B.hb.scans[s];
        const ScanState& st = B.h_state[s];
        lp_scan_output& o = outs[s];
        const size_t n = sd.n_src;
        LP_TRY(copy_d2h(ctx, o.noise_labels, b.noise + sd.src_off, n));
        LP_TRY(copy_d2h(ctx, o.seg_labels, b.out_seg + sd.src_off, n * 4));
        LP_TRY(copy_d2h(ctx, o.cluster_labels, b.out_cl + sd.src_off, n * 4));
        o.n_obstacles = st.n_obs;
        o.n_clusters = st.n_clusters;
        o.status = LP_OK;
        if (hull && st.n_clusters <= o.cluster_capacity)
            LP_TRY(copy_d2h(ctx, hoff.data() + hbase[s], b.hull_cnt + sd.cl_off, (hbase[s + 1] - hbase[s]) * 4));
    }
    if (hull)
        LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    lp_status worst = LP_OK;
    for (size_t s = 0; hull && s < S; ++s)
    {
        const ScanDev& sd = B.hb.scans[s];
        const uint32_t k = B.h_state[s].n_clusters;
        lp_scan_output& o = outs[s];
        if (k > o.cluster_capacity)
        {
            o.status = LP_ERR_CAPACITY;
            if (worst == LP_OK)
                worst = fail(ctx, LP_ERR_CAPACITY, "scan " + std::to_string(s) + ": cluster_capacity too small");
            continue;
        }
        const uint32_t* ho = hoff.data() + hbase[s];
        const uint32_t base = ho[0];
        const uint32_t nh = ho[k] - base;
        if (nh > o.hull_capacity)
        {
            o.status = LP_ERR_CAPACITY;
            if (worst == LP_OK)
                worst = fail(ctx, LP_ERR_CAPACITY, "scan " + std::to_string(s) + ": hull_capacity too small");
            continue;
        }
        if (o.hull_offsets)
            for (uint32_t i = 0; i <= k; ++i)
                o.hull_offsets[i] = ho[i] - base;
        o.n_hull_indices = nh;
        LP_TRY(copy_d2h(ctx, o.hull_indices, b.hull_out + base, static_cast<size_t>(nh) * 4));
        LP_TRY(copy_d2h(ctx, o.z_min, b.cl_zmin + sd.cl_off, static_cast<size_t>(k) * 4));
        LP_TRY(copy_d2h(ctx, o.z_max, b.cl_zmax + sd.cl_off, static_cast<size_t>(k) * 4));
        if (B.run.stages & ST_OBB)
        {
            LP_TRY(copy_d2h(ctx, o.obb_calipers, b.obb_c + sd.cl_off, static_cast<size_t>(k) * sizeof(lp_bounding_box)));
            LP_TRY(copy_d2h(ctx, o.obb_pca, b.obb_p + sd.cl_off, static_cast<size_t>(k) * sizeof(lp_bounding_box)));
        }
    }
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return worst;
}

lp_status fill_pipeline(lp_context* ctx, lp_batch& B, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                        uint32_t nscans)
{
    if (!cfg || (!scans && nscans))
        return fail(ctx, LP_ERR_BAD_ARG, "null pipeline configuration or scans");
    Run& R = B.run;
    R = Run{};
    R.stages = ST_SEG | ST_CLUSTER | ST_HULL | (cfg->compute_obb ? ST_OBB : 0u) |
               (cfg->enable_noise_removal ? ST_NOISE : 0u);
    R.cl = cfg->cluster;
    R.nr = cfg->noise;
    for (uint32_t i = 0; i < nscans; ++i)
    {
        if (scans[i].n && !scans[i].xyzi)
            return fail(ctx, LP_ERR_BAD_ARG, "scan with points but no xyzi pointer");
        ScanIn in;
        in.xyzi = scans[i].xyzi;
        in.ring = cfg->compute_ring ? nullptr : scans[i].ring;
        in.n = scans[i].n;
        in.seg = scans[i].seg;
        in.compute_ring = cfg->compute_ring;
        in.first_ring = cfg->first_ring ? static_cast<int32_t>(cfg->first_ring) : -1; // 0: image_height - 1
        R.scans.push_back(in);
    }
    return LP_OK;
}
size_t measure(lp_batch& B)
{
    return carve(B, nullptr);
}
} // namespace lprt

using namespace lprt;

// =============================================================================================
// C ABI
// =============================================================================================
namespace lprt
{
// Page-locked host allocations made by lp_host_alloc: [base, base + bytes).
std::mutex g_pin_mu;
std::map<uintptr_t, size_t> g_pinned;

bool pinned_range(const void* p, size_t bytes)
{
    if (!p)
        return true;
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    std::lock_guard<std::mutex> lk(g_pin_mu);
    auto it = g_pinned.upper_bound(a);
    if (it == g_pinned.begin())
        return false;
    --it;
    return a + bytes <= it->first + it->second;
}

// Direct host I/O applies when every buffer of the call lies in lp_host_alloc memory (inputs as
// XYZI); the GPU then reads and writes them itself over the coherent host link.
bool direct_io_ok(const lp_batch& B, const lp_scan_input* scans, const lp_scan_output* outs)
{
    const bool hull = B.run.stages & ST_HULL, obb = B.run.stages & ST_OBB;
    for (size_t s = 0; s < B.run.scans.size(); ++s)
    {
        const ScanIn& in = B.run.scans[s];
        const lp_scan_output& o = outs[s];
        const size_t n = in.n;
        if (in.n && (in.stride != 4 || !in.xyzi || !pinned_range(in.xyzi, n * 16)))
            return false;
        if (!pinned_range(in.ring, n * 2) || !pinned_range(o.noise_labels, n) || !pinned_range(o.seg_labels, n * 4) ||
            !pinned_range(o.cluster_labels, n * 4))
            return false;
        if (hull)
        {
            const size_t cc = o.cluster_capacity, hc = o.hull_capacity;
            if (!pinned_range(o.hull_offsets, (cc + 1) * 4) || !pinned_range(o.hull_indices, hc * 4) ||
                !pinned_range(o.z_min, cc * 4) || !pinned_range(o.z_max, cc * 4))
                return false;
            if (obb && (!pinned_range(o.obb_calipers, cc * sizeof(lp_bounding_box)) ||
                        !pinned_range(o.obb_pca, cc * sizeof(lp_bounding_box))))
                return false;
        }
    }
    (void)scans;
    return true;
}

// Launches of the direct host I/O path on the batch's stream: inputs gathered from the caller's
// page-locked buffers, the pipeline, results scattered into them, the scans' states read back.
lp_status direct_launch(lp_context* ctx, lp_batch& B, lp_scan_output* outs)
{
    LP_TRY(build(ctx, B));
    BatchDev& b = B.b;
    const cudaStream_t st = B.stream ? B.stream : ctx->stream;
    const size_t S = B.run.scans.size();
    const bool hull = B.run.stages & ST_HULL, obb = B.run.stages & ST_OBB;
    std::vector<IoScan> io(S);
    uint32_t nq = 0; // 4-point chunks of the batch
    auto aligned = [](const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) & (a - 1)) == 0; };
    for (size_t s = 0; s < S; ++s)
    {
        const ScanIn& in = B.run.scans[s];
        const lp_scan_output& o = outs[s];
        const uint32_t vec = aligned(o.noise_labels, 4) && aligned(o.seg_labels, 16) && aligned(o.cluster_labels, 16);
        io[s] = IoScan{in.xyzi, in.ring, o.noise_labels, o.seg_labels, o.cluster_labels,
                       hull ? o.hull_offsets : nullptr, hull ? o.hull_indices : nullptr,
                       hull ? o.z_min : nullptr, hull ? o.z_max : nullptr,
                       obb ? o.obb_calipers : nullptr, obb ? o.obb_pca : nullptr,
                       o.cluster_capacity, o.hull_capacity, nq, vec};
        nq += (in.n + 3u) / 4u;
    }
    LP_CUDA(ctx, cudaMemcpyAsync(const_cast<ScanDev*>(b.scans), B.hb.scans.data(), S * sizeof(ScanDev),
                                 cudaMemcpyHostToDevice, st));
    LP_CUDA(ctx, cudaMemcpyAsync(b.io, io.data(), S * sizeof(IoScan), cudaMemcpyHostToDevice, st));
    Launcher L;
    L.stream = st;
    L.launches = &ctx->launches;
    launch_io_in(L, b, b.io);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "direct input launch");
    LP_TRY(execute(ctx, B));
    launch_io_out(L, b, b.io, b.io_ret, hull ? 1 : 0, obb ? 1 : 0, nq);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "direct output launch");
    return LP_OK;
}

// Reads the scans' states back (a copy into pageable memory waits for the batch's stream, so it is
// issued only here, after every part of a split call has been launched) and reports every scan's
// status and counts in outs.
lp_status direct_finish(lp_context* ctx, lp_batch& B, lp_scan_output* outs)
{
    const cudaStream_t st = B.stream ? B.stream : ctx->stream;
    const size_t S = B.run.scans.size();
    const bool hull = B.run.stages & ST_HULL;
    B.h_nh.assign(S, 0u);
    const std::vector<uint32_t>& nh = B.h_nh;
    LP_CUDA(ctx, cudaMemcpyAsync(B.h_state.data(), B.b.state, S * sizeof(ScanState), cudaMemcpyDeviceToHost, st));
    if (hull)
        LP_CUDA(ctx, cudaMemcpyAsync(B.h_nh.data(), B.b.io_ret, S * 4, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    lp_status worst = report_state(ctx, B);
    if (worst != LP_OK && worst != LP_ERR_CAPACITY)
        return worst;
    for (size_t s = 0; s < S; ++s)
    {
        lp_scan_output& o = outs[s];
        const ScanState& sst = B.h_state[s];
        o.n_obstacles = sst.n_obs;
        o.n_clusters = sst.n_clusters;
        o.n_hull_indices = hull ? nh[s] : 0u;
        o.status = LP_OK;
        if (hull && (sst.n_clusters > o.cluster_capacity || nh[s] > o.hull_capacity))
        {
            o.status = LP_ERR_CAPACITY;
            o.n_hull_indices = 0;
            if (worst == LP_OK)
                worst = fail(ctx, LP_ERR_CAPACITY, "scan " + std::to_string(s) + ": cluster or hull capacity too small");
        }
    }
    return worst;
}

lp_status run_direct(lp_context* ctx, lp_batch& B, lp_scan_output* outs)
{
    LP_TRY(direct_launch(ctx, B, outs));
    return direct_finish(ctx, B, outs);
}

// The direct path for a split batch: concurrent parts (the scans the tuning assigns each), each on
// its own stream, ordered after earlier work on the context stream; each part's host reads and
// writes overlap the other parts' kernels.
lp_status run_direct_split(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                           lp_scan_output* outs, uint32_t nscans, const lp_tuning& tune, uint32_t K)
{
    const std::vector<std::vector<uint32_t>> where = assign_parts(scans, nscans, K, tune.balance_parts != 0);
    while (ctx->cached_parts.size() < K)
    {
        lp_batch* P = new lp_batch();
        if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess)
        {
            delete P;
            return fail(ctx, LP_ERR_CUDA, "cudaStreamCreateWithFlags");
        }
        ctx->cached_parts.push_back(P);
    }
    if (!ctx->fork)
        LP_CUDA(ctx, cudaEventCreateWithFlags(&ctx->fork, cudaEventDisableTiming));
    LP_CUDA(ctx, cudaEventRecord(ctx->fork, ctx->stream));
    std::vector<std::vector<lp_scan_output>> sub(K);
    lp_status worst = LP_OK;
    uint32_t launched = 0;
    for (uint32_t k = 0; k < K && worst == LP_OK; ++k)
    {
        lp_batch& P = *ctx->cached_parts[k];
        P.tune = tune;
        std::vector<lp_scan_input> in;
        for (const uint32_t i : where[k])
        {
            in.push_back(scans[i]);
            sub[k].push_back(outs[i]);
        }
        LP_CUDA(ctx, cudaStreamWaitEvent(P.stream, ctx->fork, 0));
        worst = fill_pipeline(ctx, P, cfg, in.data(), static_cast<uint32_t>(in.size()));
        if (worst == LP_OK)
            worst = direct_launch(ctx, P, sub[k].data());
        if (worst == LP_OK)
            ++launched;
    }
    if (worst != LP_OK)
    {
        for (uint32_t k = 0; k < K; ++k)
            cudaStreamSynchronize(ctx->cached_parts[k]->stream);
        return worst;
    }
    for (uint32_t k = 0; k < launched; ++k)
    {
        const lp_status st = direct_finish(ctx, *ctx->cached_parts[k], sub[k].data());
        for (size_t j = 0; j < sub[k].size(); ++j)
            outs[where[k][j]] = sub[k][j];
        if (st != LP_OK && (worst == LP_OK || worst == LP_ERR_CAPACITY))
            worst = st;
    }
    return worst;
}
lp_status create_batch(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans, uint32_t nscans,
                       const lp_tuning& tune, lp_batch** out)
{
    if (!ctx || !out || nscans == 0)
        return fail(ctx, LP_ERR_BAD_ARG, "null argument or empty batch");
    *out = nullptr;
    LP_TRY(ensure_device(ctx));
    lp_batch* B = new lp_batch();
    B->tune = tune;
    const uint32_t K = part_count(tune, nscans);
    lp_status st = LP_OK;
    if (K == 1)
    {
        st = fill_pipeline(ctx, *B, cfg, scans, nscans);
        if (st == LP_OK)
            st = build(ctx, *B);
        if (st == LP_OK)
            st = upload(ctx, *B);
    }
    else
    {
        // scans dealt round-robin (every part gets a similar mix of scan sizes) or by points
        B->part_scans = assign_parts(scans, nscans, K, tune.balance_parts != 0);
        for (uint32_t k = 0; k < K && st == LP_OK; ++k)
        {
            std::vector<lp_scan_input> sub;
            for (const uint32_t i : B->part_scans[k])
                sub.push_back(scans[i]);
            lp_batch* P = new lp_batch();
            P->tune = tune;
            B->parts.push_back(P);
            if (cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking) != cudaSuccess)
                st = fail(ctx, LP_ERR_CUDA, "cudaStreamCreateWithFlags");
            if (st == LP_OK)
                st = fill_pipeline(ctx, *P, cfg, sub.data(), static_cast<uint32_t>(sub.size()));
            if (st == LP_OK)
                st = build(ctx, *P);
            if (st == LP_OK)
                st = upload(ctx, *P);
        }
        for (uint32_t k = 0; k <= K && st == LP_OK; ++k)
        {
            cudaEvent_t e;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                st = fail(ctx, LP_ERR_CUDA, "cudaEventCreateWithFlags");
            else
                B->fork_join.push_back(e);
        }
    }
    if (st != LP_OK)
    {
        cudaStreamSynchronize(ctx->stream);
        destroy_batch(B);
        return st;
    }
    *out = B;
    return LP_OK;
}
} // namespace lprt

extern "C" {

void lp_segmenter_config_default(lp_segmenter_config* c)
{
    // SegmenterConfiguration member initialisers, segmenter.hpp:91-108
    c->elevation_up_deg = 2.0F;
    c->elevation_down_deg = -24.8F;
    c->image_width = 2048;
    c->image_height = 64;
    c->assume_unorganized_cloud = 0;
    c->grid_radial_spacing_m = 2.0F;
    c->grid_slice_resolution_deg = 1.0F;
    c->ground_height_threshold_m = 0.2F;
    c->road_maximum_slope_m_per_m = 0.2F;
    c->min_distance_m = 2.0F;
    c->max_distance_m = 100.0F;
    c->sensor_height_m = 1.73F;
    c->kernel_threshold_distance_m = 1.0F;
    c->amplification_factor = 5.0F;
    c->z_min_m = -3.0F;
    c->z_max_m = 4.0F;
}

void lp_noise_remover_config_default(lp_noise_remover_config* c)
{
    // noise_remover.hpp:41-54
    c->radius_multiplier_m_per_m = 0.02F;
    c->min_search_radius_m = 0.1F;
    c->min_neighbours = 4U;
}

void lp_clusterer_config_default(lp_clusterer_config* c)
{
    // clusterer.hpp:61-68
    c->voxel_grid_range_resolution_m = 0.4F;
    c->voxel_grid_azimuth_resolution_deg = 1.0F;
    c->voxel_grid_elevation_resolution_deg = 1.5F;
    c->min_cluster_size = 3;
}

void lp_pipeline_config_default(lp_pipeline_config* c)
{
    lp_clusterer_config_default(&c->cluster);
    c->cluster.voxel_grid_elevation_resolution_deg = 3.0F; // processor.param.yaml:34
    lp_noise_remover_config_default(&c->noise);
    c->enable_noise_removal = 0;
    c->compute_ring = 0;
    c->first_ring = 0;
    c->reserved0 = 0;
    c->compute_obb = 1;
}

const char* lp_status_string(lp_status s)
{
    switch (s)
    {
    case LP_OK:
        return "ok";
    case LP_ERR_BAD_ARG:
        return "bad argument";
    case LP_ERR_CAPACITY:
        return "capacity exceeded";
    case LP_ERR_TIMEOUT:
        return "bounded device wait timed out";
    case LP_ERR_CUDA:
        return "CUDA error";
    case LP_ERR_NO_DEVICE:
        return "no CUDA device";
    case LP_ERR_INTERNAL:
        return "internal consistency check failed";
    default:
        return "unknown status";
    }
}

lp_status lp_context_create(int32_t device, lp_context** out)
{
    if (!out)
        return LP_ERR_BAD_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    {
        cudaGetLastError();
        return LP_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count)
        return LP_ERR_BAD_ARG;
    lp_context* ctx = new lp_context();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        cudaGetLastError();
        delete ctx;
        return LP_ERR_CUDA;
    }
    init_kernel_attributes();
    init_segment_tables();
    *out = ctx;
    return LP_OK;
}

void lp_context_destroy(lp_context* ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    destroy_batch(ctx->cached);
    for (lp_batch* P : ctx->cached_parts)
    {
        cudaStreamSynchronize(P->stream);
        destroy_batch(P);
    }
    if (ctx->fork)
        cudaEventDestroy(ctx->fork);
    if (ctx->split_mem)
        cudaFree(ctx->split_mem);
    for (cudaEvent_t e : ctx->events)
        cudaEventDestroy(e);
    if (ctx->flush)
        cudaFree(ctx->flush);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* lp_last_error(const lp_context* ctx)
{
    return ctx ? ctx->last_error.c_str() : "";
}

uint64_t lp_kernel_launch_count(const lp_context* ctx)
{
    return ctx ? ctx->launches : 0;
}

namespace
{
// Device scratch of the standalone conversion entry points (grown on demand, kept by the context).
lp_status scratch(lp_context* ctx, size_t bytes, char** out)
{
    if (bytes > ctx->split_cap)
    {
        if (ctx->split_mem)
        {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(ctx->split_mem);
            ctx->split_mem = nullptr;
            ctx->split_cap = 0;
        }
        LP_CUDA(ctx, cudaMalloc(&ctx->split_mem, bytes));
        ctx->split_cap = bytes;
    }
    *out = static_cast<char*>(ctx->split_mem);
    return LP_OK;
}
} // namespace

lp_status lp_unpack_pointcloud2(lp_context* ctx, const uint8_t* data, uint32_t width, uint32_t height,
                                uint32_t point_step, uint32_t row_step, const uint32_t* offsets, float* xyzi_out,
                                uint16_t* ring_out)
{
    const uint64_t n = static_cast<uint64_t>(width) * height;
    if (!ctx || !offsets || (n && (!data || !xyzi_out)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (n == 0)
        return LP_OK;
    if (n > 0x7fffffffull / 4)
        return fail(ctx, LP_ERR_CAPACITY, "cloud too large for 32-bit indexing");
    const uint64_t need = static_cast<uint64_t>(width - 1) * point_step + point_step;
    // every field inside the point record (64-bit sums: no offset can wrap past the check)
    auto fits = [&](uint32_t off, uint64_t size) { return static_cast<uint64_t>(off) + size <= point_step; };
    bool ok = point_step > 0 && row_step >= need && fits(offsets[0], 4) && fits(offsets[1], 4) && fits(offsets[2], 4);
    ok = ok && (offsets[3] == LP_NO_FIELD || fits(offsets[3], 4));
    ok = ok && (offsets[4] == LP_NO_FIELD || fits(offsets[4], 2));
    if (!ok)
        return fail(ctx, LP_ERR_BAD_ARG, "field offsets or steps outside the point record");
    LP_TRY(ensure_device(ctx));
    auto al = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
    const size_t in_bytes = static_cast<size_t>(row_step) * height;
    const size_t o_xyzi = al(in_bytes), o_ring = o_xyzi + al(n * 16);
    char* m = nullptr;
    LP_TRY(scratch(ctx, o_ring + al(n * 2), &m));
    const cudaStream_t st = ctx->stream;
    LP_CUDA(ctx, cudaMemcpyAsync(m, data, in_bytes, cudaMemcpyHostToDevice, st));
    launch_unpack_pointcloud2(st, reinterpret_cast<const uint8_t*>(m), width, height, point_step, row_step, offsets,
                              reinterpret_cast<float4*>(m + o_xyzi),
                              ring_out ? reinterpret_cast<uint16_t*>(m + o_ring) : nullptr, ctx->launches);
    LP_CUDA(ctx, cudaGetLastError());
    LP_CUDA(ctx, cudaMemcpyAsync(xyzi_out, m + o_xyzi, n * 16, cudaMemcpyDeviceToHost, st));
    if (ring_out)
        LP_CUDA(ctx, cudaMemcpyAsync(ring_out, m + o_ring, n * 2, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    return LP_OK;
}

lp_status lp_split_clouds(lp_context* ctx, const float* xyzi, const uint32_t* labels, uint32_t n, lp_xyzrgb* ground,
                          lp_xyzrgb* obstacle, lp_xyzrgb* unsegmented, uint32_t* counts)
{
    if (!ctx || !counts || (n && (!xyzi || !labels)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    counts[0] = counts[1] = counts[2] = 0;
    if (n == 0)
        return LP_OK;
    if (n > 0x7fffffffu / 4u)
        return fail(ctx, LP_ERR_CAPACITY, "cloud too large for 32-bit indexing");
    LP_TRY(ensure_device(ctx));
    auto al = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
    const size_t N = n;
    const size_t o_lab = al(N * 16), o_out = o_lab + al(N * 4), o_cnt = o_out + al(3 * N * sizeof(lp_xyzrgb));
    const size_t o_sums = o_cnt + 256;
    char* m = nullptr;
    LP_TRY(scratch(ctx, o_sums + al((N + 1) / 8192 * 8 + 64), &m));
    const cudaStream_t st = ctx->stream;
    LP_CUDA(ctx, cudaMemcpyAsync(m, xyzi, N * 16, cudaMemcpyHostToDevice, st));
    LP_CUDA(ctx, cudaMemcpyAsync(m + o_lab, labels, N * 4, cudaMemcpyHostToDevice, st));
    lp_xyzrgb* out = reinterpret_cast<lp_xyzrgb*>(m + o_out);
    uint32_t* dcnt = reinterpret_cast<uint32_t*>(m + o_cnt);
    launch_split_clouds(st, reinterpret_cast<const float4*>(m), reinterpret_cast<const uint32_t*>(m + o_lab), n, out, dcnt,
                        reinterpret_cast<uint32_t*>(m + o_sums), ctx->launches);
    LP_CUDA(ctx, cudaGetLastError());
    LP_CUDA(ctx, cudaMemcpyAsync(counts, dcnt, 3 * 4, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    lp_xyzrgb* dst[3] = {ground, obstacle, unsegmented};
    for (int c = 0; c < 3; ++c)
        if (dst[c] && counts[c])
            LP_CUDA(ctx, cudaMemcpyAsync(dst[c], out + static_cast<size_t>(c) * N, counts[c] * sizeof(lp_xyzrgb),
                                         cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    return LP_OK;
}

namespace
{
// processor.hpp:60-192: vehicle types widened by the tolerances, their volume and area bounds and
// the overall limits, in the same binary64 expressions (host code is built without contraction).
VehicleTableDev vehicle_table()
{
    VehicleTableDev t{};
    const double base[5][6] = {{4.3, 4.6, 1.6, 1.9, 1.4, 1.5},
                                {4.6, 5.0, 1.6, 1.9, 1.4, 1.5},
                                {4.6, 5.2, 1.7, 2.1, 1.7, 1.8},
                                {5.2, 5.8, 1.9, 2.2, 1.8, 2.0},
                                {4.9, 5.2, 1.7, 2.1, 1.7, 1.8}};
    const double lt = 0.8, wt = 0.5, ht = 0.5;
    for (int v = 0; v < 5; ++v)
    {
        t.dims[v][0] = base[v][0] - lt;
        t.dims[v][1] = base[v][1] + lt;
        t.dims[v][2] = base[v][2] - wt;
        t.dims[v][3] = base[v][3] + wt;
        t.dims[v][4] = base[v][4] - ht;
        t.dims[v][5] = base[v][5] + ht;
        t.bounds[v][0] = t.dims[v][0] * t.dims[v][2] * t.dims[v][4];
        t.bounds[v][1] = t.dims[v][1] * t.dims[v][3] * t.dims[v][5];
        t.bounds[v][2] = t.dims[v][0] * t.dims[v][2];
        t.bounds[v][3] = t.dims[v][1] * t.dims[v][3];
    }
    t.min_h = std::numeric_limits<double>::max();
    t.max_h = std::numeric_limits<double>::lowest();
    t.min_v = std::numeric_limits<double>::max();
    t.max_v = std::numeric_limits<double>::lowest();
    for (int v = 0; v < 5; ++v)
    {
        t.min_h = std::min(t.min_h, t.dims[v][4]);
        t.max_h = std::max(t.max_h, t.dims[v][5]);
        t.min_v = std::min(t.min_v, t.bounds[v][0]);
        t.max_v = std::max(t.max_v, t.bounds[v][1]);
    }
    return t;
}

// glibc rand() (TYPE_3 additive feedback generator, the state rand() uses when never seeded):
// r[0] = 1, r[i] = 16807 r[i-1] mod (2^31 - 1) for i < 31, r[31..33] = r[0..2], then
// r[i] = r[i-31] + r[i-3] mod 2^32 with 310 values discarded; rand() returns r[i] >> 1. The window
// holds the last 34 values; `draws` values are skipped (advanced from the context's cached window
// when it lies behind).
void rand_step(RandWindow& w)
{
    w.r[w.pos] = w.r[(w.pos + 3u) % 34u] + w.r[(w.pos + 31u) % 34u];
    w.pos = (w.pos + 1u) % 34u;
}

RandWindow rand_window(lp_context* ctx, uint64_t draws)
{
    if (!ctx->rand_valid || draws < ctx->rand_at)
    {
        RandWindow w{};
        int64_t word = 1;
        w.r[0] = 1u;
        for (int k = 1; k < 31; ++k)
        {
            const int64_t hi = word / 127773, lo = word % 127773;
            word = 16807 * lo - 2836 * hi;
            if (word < 0)
                word += 2147483647;
            w.r[k] = static_cast<uint32_t>(word);
        }
        for (int k = 31; k < 34; ++k)
            w.r[k] = w.r[k - 31];
        w.pos = 0; // slot of r[34] (index 34 mod 34)
        for (int k = 0; k < 310; ++k)
            rand_step(w);
        ctx->rand_window = w;
        ctx->rand_at = 0;
        ctx->rand_valid = true;
    }
    for (; ctx->rand_at < draws; ++ctx->rand_at)
        rand_step(ctx->rand_window);
    return ctx->rand_window;
}
} // namespace

lp_status lp_cluster_objects(lp_context* ctx, const float* xyzi, const int32_t* cluster_labels, uint32_t n,
                             uint32_t n_clusters, const uint32_t* hull_offsets, const int32_t* hull_indices,
                             const float* z_min, const float* z_max, const lp_object_config* cfg,
                             lp_object_output* out)
{
    if (!ctx || !cfg || !out || (n && (!xyzi || !cluster_labels)) ||
        (n_clusters && (!hull_offsets || !z_min || !z_max)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    out->n_clustered = 0;
    out->n_marker_points = 0;
    const uint32_t K = n_clusters;
    if (K && out->marker_offsets)
        std::memset(out->marker_offsets, 0, (static_cast<size_t>(K) + 1) * 4);
    if (K == 0)
    {
        if (out->marker_offsets)
            out->marker_offsets[0] = 0;
        return LP_OK;
    }
    if (hull_offsets[0] != 0)
        return fail(ctx, LP_ERR_BAD_ARG, "hull_offsets[0] must be 0");
    for (uint32_t l = 0; l < K; ++l)
        if (hull_offsets[l + 1] < hull_offsets[l])
            return fail(ctx, LP_ERR_BAD_ARG, "hull_offsets must not decrease");
    const uint32_t H = hull_offsets[K];
    if (H && !hull_indices)
        return fail(ctx, LP_ERR_BAD_ARG, "null hull_indices");
    if (n > 0x7fffffffu / 8u)
        return fail(ctx, LP_ERR_CAPACITY, "cloud too large for 32-bit indexing");
    const uint32_t ntiles = obj_tiles(n);
    const uint64_t cells = static_cast<uint64_t>(K) * ntiles + 1;
    if (cells > 0x7fffffffull)
        return fail(ctx, LP_ERR_CAPACITY, "too many clusters for the cloud's size");
    const uint64_t mcap = 6ull * (static_cast<uint64_t>(H) + 4ull * K); // a polygon has max(h, 4) points
    if (mcap > 0x7fffffffull)
        return fail(ctx, LP_ERR_CAPACITY, "marker geometry too large");
    LP_TRY(ensure_device(ctx));
    auto al = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
    const size_t N = n;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += al(std::max<size_t>(bytes, 1));
        return at;
    };
    const size_t o_pts = take(N * 16), o_lab = take(N * 4), o_cnt = take(cells * 4),
                 o_sums = take(8 * (cells / 2048 + 4)), o_err = take(4), o_col = take(static_cast<size_t>(K) * 4),
                 o_cloff = take((K + 1ull) * 4), o_cloud = take(N * sizeof(lp_xyzrgb)), o_hoff = take((K + 1ull) * 4),
                 o_hidx = take(static_cast<size_t>(H) * 4), o_zmin = take(K * 4ull), o_zmax = take(K * 4ull),
                 o_cls = take(K * 4ull), o_box = take(K * sizeof(lp_bounding_box)), o_P = take(N * 16),
                 o_Pf = take(N * 8), o_ea = take(N * 4), o_pairs = take((4ull * N + 16ull * K) * 8),
                 o_state = take(sizeof(ScanState)), o_moff = take((K + 1ull) * 4), o_mpts = take(mcap * 24);
    char* m = nullptr;
    LP_TRY(scratch(ctx, o, &m));
    const cudaStream_t st = ctx->stream;
    if (n)
    {
        LP_CUDA(ctx, cudaMemcpyAsync(m + o_pts, xyzi, N * 16, cudaMemcpyHostToDevice, st));
        LP_CUDA(ctx, cudaMemcpyAsync(m + o_lab, cluster_labels, N * 4, cudaMemcpyHostToDevice, st));
    }
    LP_CUDA(ctx, cudaMemcpyAsync(m + o_hoff, hull_offsets, (K + 1ull) * 4, cudaMemcpyHostToDevice, st));
    if (H)
        LP_CUDA(ctx, cudaMemcpyAsync(m + o_hidx, hull_indices, static_cast<size_t>(H) * 4, cudaMemcpyHostToDevice, st));
    LP_CUDA(ctx, cudaMemcpyAsync(m + o_zmin, z_min, K * 4ull, cudaMemcpyHostToDevice, st));
    LP_CUDA(ctx, cudaMemcpyAsync(m + o_zmax, z_max, K * 4ull, cudaMemcpyHostToDevice, st));
    LP_CUDA(ctx, cudaMemsetAsync(m + o_cnt, 0, cells * 4, st));
    LP_CUDA(ctx, cudaMemsetAsync(m + o_err, 0, 4, st));
    LP_CUDA(ctx, cudaMemsetAsync(m + o_state, 0, sizeof(ScanState), st));
    const RandWindow w = rand_window(ctx, cfg->rand_draws);
    uint32_t* err = reinterpret_cast<uint32_t*>(m + o_err);
    uint32_t* sums = reinterpret_cast<uint32_t*>(m + o_sums);
    auto* cloud = reinterpret_cast<lp_xyzrgb*>(m + o_cloud);
    launch_objects_cloud(st, reinterpret_cast<const float4*>(m + o_pts), reinterpret_cast<const int32_t*>(m + o_lab), n, K,
                         reinterpret_cast<uint32_t*>(m + o_cnt), sums, err, w, reinterpret_cast<uchar4*>(m + o_col),
                         reinterpret_cast<uint32_t*>(m + o_cloff), cloud, ctx->launches);
    ObjDev od{};
    od.K = K;
    od.cl_off = reinterpret_cast<const uint32_t*>(m + o_cloff);
    od.hull_off = reinterpret_cast<const uint32_t*>(m + o_hoff);
    od.hull_idx = reinterpret_cast<const int32_t*>(m + o_hidx);
    od.zmin = reinterpret_cast<const float*>(m + o_zmin);
    od.zmax = reinterpret_cast<const float*>(m + o_zmax);
    od.cls = reinterpret_cast<int32_t*>(m + o_cls);
    od.boxes = reinterpret_cast<lp_bounding_box*>(m + o_box);
    od.cloud = cloud;
    od.moff = reinterpret_cast<uint32_t*>(m + o_moff);
    od.mpts = reinterpret_cast<double*>(m + o_mpts);
    od.mcap = static_cast<uint32_t>(mcap);
    static const VehicleTableDev vt = vehicle_table();
    launch_objects_gates(st, od, vt, cfg->vehicle_gates, reinterpret_cast<double2*>(m + o_P),
                         reinterpret_cast<float2*>(m + o_Pf), reinterpret_cast<float*>(m + o_ea),
                         reinterpret_cast<int2*>(m + o_pairs), reinterpret_cast<ScanState*>(m + o_state),
                         ctx->launches);
    launch_objects_markers(st, od, sums, ctx->launches);
    LP_CUDA(ctx, cudaGetLastError());
    uint32_t h_err = 0, h_nc = 0, h_nm = 0;
    ScanState h_state{};
    LP_CUDA(ctx, cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaMemcpyAsync(&h_nc, m + o_cloff + 4ull * K, 4, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaMemcpyAsync(&h_nm, m + o_moff + 4ull * K, 4, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaMemcpyAsync(&h_state, m + o_state, sizeof(ScanState), cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    if (h_err)
        return fail(ctx, LP_ERR_BAD_ARG, "a cluster label is not below n_clusters");
    if (h_state.err)
        return fail(ctx, LP_ERR_INTERNAL, "vehicle gate: calipers pair capacity exceeded");
    out->n_clustered = h_nc;
    out->n_marker_points = h_nm;
    if (out->clustered_cloud && h_nc)
        LP_CUDA(ctx, cudaMemcpyAsync(out->clustered_cloud, cloud, h_nc * sizeof(lp_xyzrgb), cudaMemcpyDeviceToHost, st));
    if (out->vehicle_class)
        LP_CUDA(ctx, cudaMemcpyAsync(out->vehicle_class, m + o_cls, K * 4ull, cudaMemcpyDeviceToHost, st));
    if (out->gate_boxes)
        LP_CUDA(ctx, cudaMemcpyAsync(out->gate_boxes, m + o_box, K * sizeof(lp_bounding_box), cudaMemcpyDeviceToHost, st));
    if (out->marker_offsets)
        LP_CUDA(ctx, cudaMemcpyAsync(out->marker_offsets, m + o_moff, (K + 1ull) * 4, cudaMemcpyDeviceToHost, st));
    const bool fits = h_nm <= out->marker_capacity;
    if (out->marker_points && h_nm && fits)
        LP_CUDA(ctx, cudaMemcpyAsync(out->marker_points, m + o_mpts, h_nm * 24ull, cudaMemcpyDeviceToHost, st));
    LP_CUDA(ctx, cudaStreamSynchronize(st));
    if (out->marker_points && !fits)
        return fail(ctx, LP_ERR_CAPACITY, "marker_capacity below n_marker_points");
    return LP_OK;
}

lp_status lp_add_ring_info(lp_context* ctx, const float* xyzi, uint32_t n, uint16_t first_ring, uint16_t* ring_out)
{
    if (!ctx || (n && (!xyzi || !ring_out)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (n == 0)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    B.run = Run{};
    B.run.stages = ST_RING;
    ScanIn in;
    in.xyzi = xyzi;
    in.n = n;
    in.compute_ring = 1;
    in.first_ring = first_ring;
    B.run.scans.push_back(in);
    LP_TRY(run_once(ctx, B));
    LP_CUDA(ctx, cudaMemcpyAsync(ring_out, B.b.ring, static_cast<size_t>(n) * 2, cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

lp_status lp_segment(lp_context* ctx, const float* xyzi, const uint16_t* ring, uint32_t n,
                     const lp_segmenter_config* cfg, uint32_t* labels_out, uint8_t* image_bgr_out)
{
    if (!ctx || !cfg || (n && (!xyzi || !labels_out)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (!seg_config_ok(*cfg))
        return fail(ctx, LP_ERR_BAD_ARG, "segmenter configuration out of the supported range");
    if (n == 0 && !image_bgr_out)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    B.run = Run{};
    B.run.stages = ST_SEG | (image_bgr_out ? ST_IMAGE : 0u);
    ScanIn in;
    in.xyzi = xyzi;
    in.ring = ring;
    in.n = n;
    in.seg = *cfg;
    B.run.scans.push_back(in);
    LP_TRY(run_once(ctx, B));
    LP_TRY(copy_d2h(ctx, labels_out, B.b.out_seg, static_cast<size_t>(n) * 4));
    if (image_bgr_out)
        LP_TRY(copy_d2h(ctx, image_bgr_out, B.d_image, static_cast<size_t>(B.b.npix) * 3));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

lp_status lp_noise_remove(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n,
                          const lp_noise_remover_config* cfg, uint8_t* labels_out)
{
    if (!ctx || !cfg || (n && (!xyz || !labels_out)) || stride < 3)
        return fail(ctx, LP_ERR_BAD_ARG, "null argument or stride < 3");
    if (n == 0)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    B.run = Run{};
    B.run.stages = ST_NOISE;
    B.run.nr = *cfg;
    ScanIn in;
    in.xyzi = xyz;
    in.stride = stride;
    in.n = n;
    B.run.scans.push_back(in);
    LP_TRY(run_once(ctx, B));
    LP_TRY(copy_d2h(ctx, labels_out, B.b.noise, n));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

lp_status lp_debug_kdtree(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n,
                          const lp_noise_remover_config* cfg, float* nodes_out)
{
    if (!ctx || !cfg || (n && (!xyz || !nodes_out)) || stride < 3)
        return fail(ctx, LP_ERR_BAD_ARG, "null argument or stride < 3");
    if (n == 0)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    B.run = Run{};
    B.run.stages = ST_NOISE;
    B.run.nr = *cfg;
    ScanIn in;
    in.xyzi = xyz;
    in.stride = stride;
    in.n = n;
    B.run.scans.push_back(in);
    LP_TRY(run_once(ctx, B));
    LP_CUDA(ctx, cudaMemcpyAsync(nodes_out, B.b.kt, static_cast<size_t>(n) * sizeof(float4), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

lp_status lp_cluster(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n, const lp_clusterer_config* cfg,
                     int32_t* labels_out)
{
    if (!ctx || !cfg || (n && (!xyz || !labels_out)) || stride < 3)
        return fail(ctx, LP_ERR_BAD_ARG, "null argument or stride < 3");
    if (n == 0)
        return LP_OK;
    if (!(cfg->voxel_grid_range_resolution_m > 0) || !(cfg->voxel_grid_azimuth_resolution_deg > 0) ||
        !(cfg->voxel_grid_elevation_resolution_deg > 0))
        return fail(ctx, LP_ERR_BAD_ARG, "voxel resolution must be positive");
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    B.run = Run{};
    B.run.stages = ST_ALL_OBS;
    B.run.cl = *cfg;
    ScanIn in;
    in.xyzi = xyz;
    in.stride = stride;
    in.n = n;
    B.run.scans.push_back(in);
    LP_TRY(run_once(ctx, B));
    LP_TRY(copy_d2h(ctx, labels_out, B.b.out_cl, static_cast<size_t>(n) * 4));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

// Single-polygon entry points use a small scratch allocation of their own.
static lp_status poly_scratch(lp_context* ctx, size_t bytes, char** out)
{
    lp_batch& B = cached(ctx);
    if (B.cap < bytes)
    {
        if (B.graph)
        {
            cudaGraphExecDestroy(B.graph);
            B.graph = nullptr;
        }
        if (B.mem)
        {
            cudaStreamSynchronize(ctx->stream);
            cudaFree(B.mem);
        }
        B.mem = nullptr;
        B.cap = 0;
        LP_CUDA(ctx, cudaMalloc(reinterpret_cast<void**>(&B.mem), bytes));
        B.cap = bytes;
    }
    *out = B.mem;
    return LP_OK;
}

lp_status lp_convex_hull(lp_context* ctx, const double* xy, uint32_t n, int32_t* indices_out, uint32_t* n_out)
{
    if (!ctx || !n_out || (n && (!xy || !indices_out)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (n < 3)
    {
        // polygonizer.cpp:36-41
        for (uint32_t i = 0; i < n; ++i)
            indices_out[i] = static_cast<int32_t>(i);
        *n_out = n;
        return LP_OK;
    }
    LP_TRY(ensure_device(ctx));
    const size_t np2 = next_pow2(n);
    const size_t bytes = 4096 + n * 16 + np2 * 24 + (2 * n + 8) * 4 + (n + 8) * 4 + 64;
    char* m;
    LP_TRY(poly_scratch(ctx, bytes, &m));
    Carver c{m};
    double2* pts = c.take<double2>(n);
    char* scratch = c.take<char>(np2 * 24);
    int* stack = c.take<int>(2 * n + 8);
    int32_t* out = c.take<int32_t>(n + 8);
    uint32_t* nout = c.take<uint32_t>(4);
    LP_CUDA(ctx, cudaMemcpyAsync(pts, xy, static_cast<size_t>(n) * 16, cudaMemcpyHostToDevice, ctx->stream));
    Launcher L;
    L.stream = ctx->stream;
    L.launches = &ctx->launches;
    launch_hull_single(L, pts, n, scratch, stack, out, nout);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "lp_convex_hull launch");
    uint32_t h = 0;
    LP_CUDA(ctx, cudaMemcpyAsync(&h, nout, 4, cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    LP_CUDA(ctx, cudaMemcpyAsync(indices_out, out, static_cast<size_t>(h) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *n_out = h;
    return LP_OK;
}

static lp_status boxes_single(lp_context* ctx, const double* hull_xy, uint32_t n, int kind, lp_bounding_box* out,
                              int32_t* pairs_out, uint32_t capacity, uint32_t* n_pairs)
{
    LP_TRY(ensure_device(ctx));
    const int cap = static_cast<int>(4 * n + 16);
    const size_t bytes = 4096 + static_cast<size_t>(n) * 16 + static_cast<size_t>(cap) * 8 + sizeof(lp_bounding_box) + 64;
    char* m;
    LP_TRY(poly_scratch(ctx, bytes, &m));
    Carver c{m};
    double2* P = c.take<double2>(n + 1);
    int2* pairs = c.take<int2>(cap);
    lp_bounding_box* box = c.take<lp_bounding_box>(1);
    int* np = c.take<int>(4);
    if (n)
        LP_CUDA(ctx, cudaMemcpyAsync(P, hull_xy, static_cast<size_t>(n) * 16, cudaMemcpyHostToDevice, ctx->stream));
    Launcher L;
    L.stream = ctx->stream;
    L.launches = &ctx->launches;
    launch_boxes_single(L, P, n, pairs, cap, kind, box, np);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "bounding box launch");
    int hnp = 0;
    LP_CUDA(ctx, cudaMemcpyAsync(&hnp, np, 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (out)
        LP_CUDA(ctx, cudaMemcpyAsync(out, box, sizeof(lp_bounding_box), cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (n_pairs)
        *n_pairs = static_cast<uint32_t>(hnp);
    if (pairs_out)
    {
        if (static_cast<uint32_t>(hnp) > capacity || hnp > cap)
            return fail(ctx, LP_ERR_CAPACITY, "antipodal pair capacity too small");
        LP_CUDA(ctx, cudaMemcpyAsync(pairs_out, pairs, static_cast<size_t>(hnp) * 8, cudaMemcpyDeviceToHost, ctx->stream));
        LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return LP_OK;
}

lp_status lp_antipodal_pairs(lp_context* ctx, const double* hull_xy, uint32_t n, int32_t* pairs_out, uint32_t capacity,
                             uint32_t* n_pairs)
{
    if (!ctx || !n_pairs || (n && (!hull_xy || !pairs_out)))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (n < 2)
    {
        *n_pairs = 0;
        return LP_OK;
    }
    return boxes_single(ctx, hull_xy, n, 2, nullptr, pairs_out, capacity, n_pairs);
}

lp_status lp_bounding_box_rotating_calipers(lp_context* ctx, const double* hull_xy, uint32_t n, lp_bounding_box* out)
{
    if (!ctx || !out || (n && !hull_xy))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    std::memset(out, 0, sizeof(*out));
    if (n < 3)
        return LP_OK;
    return boxes_single(ctx, hull_xy, n, 0, out, nullptr, 0, nullptr);
}

lp_status lp_bounding_box_pca(lp_context* ctx, const double* hull_xy, uint32_t n, lp_bounding_box* out)
{
    if (!ctx || !out || (n && !hull_xy))
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    std::memset(out, 0, sizeof(*out));
    if (n < 3)
        return LP_OK;
    return boxes_single(ctx, hull_xy, n, 1, out, nullptr, 0, nullptr);
}

lp_status lp_process_batch(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                           lp_scan_output* outs, uint32_t nscans)
{
    if (!ctx || !outs)
        return fail(ctx, LP_ERR_BAD_ARG, "null argument");
    if (nscans == 0)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    lp_batch& B = cached(ctx);
    LP_TRY(fill_pipeline(ctx, B, cfg, scans, nscans));
    const lp_tuning tune = tuning_for(ctx, scans, nscans);
    B.tune = tune;
    if (direct_io_ok(B, scans, outs))
    {
        const uint32_t K = part_count(tune, nscans);
        return K > 1 ? run_direct_split(ctx, cfg, scans, outs, nscans, tune, K) : run_direct(ctx, B, outs);
    }
    const lp_status st = run_once(ctx, B);
    if (st != LP_OK && st != LP_ERR_CAPACITY)
        return st;
    const lp_status dl = download(ctx, B, outs);
    return st != LP_OK ? st : dl;
}

lp_status lp_process_scan(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scan,
                          lp_scan_output* out)
{
    return lp_process_batch(ctx, cfg, scan, out, 1);
}

// ---------------------------------------------------------------------------------------------
// Prepared batches (lidar_gb300_batch.h)
// ---------------------------------------------------------------------------------------------
lp_status lp_batch_create(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans, uint32_t nscans,
                          lp_batch** out)
{
    return create_batch(ctx, cfg, scans, nscans, tuning_for(ctx, scans, nscans), out);
}

lp_status lp_batch_create_tuned(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scans,
                                uint32_t nscans, const lp_tuning* tuning, lp_batch** out)
{
    if (!tuning || lp_tuning_validate(tuning) != LP_OK)
        return fail(ctx, LP_ERR_BAD_ARG, "tuning out of range");
    return create_batch(ctx, cfg, scans, nscans, *tuning, out);
}

lp_status lp_batch_get_tuning(const lp_batch* batch, lp_tuning* out)
{
    if (!batch || !out)
        return LP_ERR_BAD_ARG;
    *out = batch->tune;
    return LP_OK;
}

void lp_batch_destroy(lp_context* ctx, lp_batch* batch)
{
    if (ctx)
    {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    destroy_batch(batch);
}

lp_status lp_batch_upload(lp_context* ctx, lp_batch* B)
{
    if (!ctx || !B)
        return LP_ERR_BAD_ARG;
    if (B->parts.empty())
        return upload(ctx, *B);
    for (lp_batch* P : B->parts)
        LP_TRY(upload(ctx, *P));
    return LP_OK;
}

lp_status lp_batch_execute(lp_context* ctx, lp_batch* B)
{
    if (!ctx || !B)
        return LP_ERR_BAD_ARG;
    if (B->graph)
    {
        LP_CUDA(ctx, cudaGraphLaunch(B->graph, ctx->stream));
        ctx->launches += 1;
        return LP_OK;
    }
    return launch_batch(ctx, *B);
}

lp_status lp_batch_capture_graph(lp_context* ctx, lp_batch* B)
{
    if (!ctx || !B)
        return LP_ERR_BAD_ARG;
    if (B->graph)
        return LP_OK;
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    cudaGraph_t g;
    LP_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const uint64_t before = ctx->launches;
    const lp_status st = launch_batch(ctx, *B);
    const cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    ctx->launches = before;
    if (st != LP_OK)
        return st;
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamEndCapture");
    const cudaError_t ie = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess)
        return cuda_fail(ctx, ie, "cudaGraphInstantiate");
    return LP_OK;
}

lp_status lp_batch_download(lp_context* ctx, lp_batch* B, lp_scan_output* outs)
{
    if (!ctx || !B || !outs)
        return LP_ERR_BAD_ARG;
    if (!B->parts.empty())
    {
        // each part's scans in their batch order; a part's status is that of its worst scan
        const size_t K = B->parts.size();
        lp_status worst = LP_OK;
        for (size_t k = 0; k < K; ++k)
        {
            const std::vector<uint32_t>& where = B->part_scans[k];
            const size_t S = where.size();
            std::vector<lp_scan_output> sub(S);
            for (size_t j = 0; j < S; ++j)
                sub[j] = outs[where[j]];
            const lp_status st = lp_batch_download(ctx, B->parts[k], sub.data());
            for (size_t j = 0; j < S; ++j)
                outs[where[j]] = sub[j];
            if (st != LP_OK && (worst == LP_OK || worst == LP_ERR_CAPACITY))
                worst = st;
        }
        return worst;
    }
    const lp_status st = fetch_state(ctx, *B);
    if (st != LP_OK && st != LP_ERR_CAPACITY)
        return st;
    const lp_status dl = download(ctx, *B, outs);
    return st != LP_OK ? st : dl;
}

lp_status lp_context_synchronize(lp_context* ctx)
{
    if (!ctx)
        return LP_ERR_BAD_ARG;
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

uint32_t lp_batch_points(const lp_batch* B)
{
    if (!B)
        return 0;
    uint32_t n = B->b.nsrc;
    for (const lp_batch* P : B->parts)
        n += P->b.nsrc;
    return n;
}

uint64_t lp_batch_device_bytes(const lp_batch* B)
{
    if (!B)
        return 0;
    uint64_t n = B->cap;
    for (const lp_batch* P : B->parts)
        n += P->cap;
    return n;
}

// Device time of `iters` executions with CUDA events on the context stream. flush_l2: write a
// buffer larger than L2 before each execution (outside the timed interval).
lp_status lp_batch_time(lp_context* ctx, lp_batch* B, uint32_t iters, int32_t flush_l2, float* ms_per_iter)
{
    if (!ctx || !B || !ms_per_iter || iters == 0)
        return LP_ERR_BAD_ARG;
    if (flush_l2 && !ctx->flush)
    {
        ctx->flush_bytes = 512ull << 20;
        LP_CUDA(ctx, cudaMalloc(&ctx->flush, ctx->flush_bytes));
    }
    cudaEvent_t e0, e1;
    LP_CUDA(ctx, cudaEventCreate(&e0));
    LP_CUDA(ctx, cudaEventCreate(&e1));
    float total = 0.0f;
    for (uint32_t it = 0; it < iters; ++it)
    {
        if (flush_l2)
            LP_CUDA(ctx, cudaMemsetAsync(ctx->flush, static_cast<int>(it & 0xff), ctx->flush_bytes, ctx->stream));
        LP_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
        const lp_status st = lp_batch_execute(ctx, B);
        if (st != LP_OK)
            return st;
        LP_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
        LP_CUDA(ctx, cudaEventSynchronize(e1));
        float ms = 0.0f;
        LP_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
        total += ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_iter = total / static_cast<float>(iters);
    return LP_OK;
}

// Per-kernel device time of one (non-graph) execution: every launch bracketed by events on the
// context stream. Writes up to `cap` (name, milliseconds) records; *count receives the total.
lp_status lp_batch_profile(lp_context* ctx, lp_batch* B, char* names, uint32_t name_len, float* ms, uint32_t cap,
                           uint32_t* count)
{
    if (!ctx || !B || !count)
        return LP_ERR_BAD_ARG;
    // a split batch: its parts one after the other (each on its own stream, alone on the device)
    std::vector<lp_batch*> runs = B->parts;
    if (runs.empty())
        runs.push_back(B);
    uint32_t k = 0;
    for (lp_batch* P : runs)
    {
        P->prof.clear();
        P->profiling = true;
        const lp_status st = execute(ctx, *P);
        P->profiling = false;
        if (st != LP_OK)
            return st;
        LP_CUDA(ctx, cudaStreamSynchronize(P->stream ? P->stream : ctx->stream));
        for (uint32_t i = 0; i < P->prof.size(); ++i, ++k)
        {
            if (k >= cap)
                continue;
            float t = 0.0f;
            cudaEventElapsedTime(&t, P->prof[i].start, P->prof[i].stop);
            if (ms)
                ms[k] = t;
            if (names && name_len)
            {
                std::strncpy(names + static_cast<size_t>(k) * name_len, P->prof[i].name, name_len - 1);
                names[static_cast<size_t>(k) * name_len + name_len - 1] = 0;
            }
        }
    }
    *count = k;
    return LP_OK;
}

// Evaluates the device's correctly rounded binary32 functions (kind 0 atan2, 1 atan, 2 exp,
// 3 the reference's atan2 approximation) on host arrays; used by the parity tests.
lp_status lp_debug_wait_timeout(lp_context* ctx, int32_t kind, uint32_t limit, uint32_t* gave_up)
{
    if (!ctx || !gave_up || (kind != 0 && kind != 1) || limit == 0)
        return fail(ctx, LP_ERR_BAD_ARG, "kind 0 or 1, limit > 0, non-null result");
    *gave_up = 0;
    LP_TRY(ensure_device(ctx));
    char* m = nullptr;
    LP_TRY(scratch(ctx, 256, &m));
    uint32_t* err = reinterpret_cast<uint32_t*>(m + 64);
    LP_CUDA(ctx, cudaMemsetAsync(m, 0, 256, ctx->stream));
    launch_debug_wait_timeout(ctx->stream, kind, limit, reinterpret_cast<unsigned long long*>(m), err, ctx->launches);
    LP_CUDA(ctx, cudaGetLastError());
    LP_CUDA(ctx, cudaMemcpyAsync(gave_up, err, 4, cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return *gave_up ? LP_ERR_TIMEOUT : LP_OK;
}

lp_status lp_debug_math(lp_context* ctx, int32_t kind, const float* a, const float* b, uint32_t n, float* out)
{
    if (!ctx || !a || !out)
        return LP_ERR_BAD_ARG;
    if (n == 0)
        return LP_OK;
    LP_TRY(ensure_device(ctx));
    char* m;
    LP_TRY(poly_scratch(ctx, static_cast<size_t>(n) * 12 + 1024, &m));
    Carver c{m};
    float* da = c.take<float>(n);
    float* db = c.take<float>(n);
    float* dout = c.take<float>(n);
    LP_CUDA(ctx, cudaMemcpyAsync(da, a, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, ctx->stream));
    LP_CUDA(ctx, cudaMemcpyAsync(db, b ? b : a, static_cast<size_t>(n) * 4, cudaMemcpyHostToDevice, ctx->stream));
    Launcher L;
    L.stream = ctx->stream;
    L.launches = &ctx->launches;
    launch_debug_math(L, kind, da, db, n, dout);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "lp_debug_math launch");
    LP_CUDA(ctx, cudaMemcpyAsync(out, dout, static_cast<size_t>(n) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return LP_OK;
}

lp_status lp_host_alloc(uint64_t bytes, void** out)
{
    if (!out)
        return LP_ERR_BAD_ARG;
    *out = nullptr;
    if (bytes == 0)
        return LP_OK;
    if (cudaMallocHost(out, static_cast<size_t>(bytes)) != cudaSuccess)
    {
        cudaGetLastError();
        *out = nullptr;
        return LP_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lk(lprt::g_pin_mu);
    lprt::g_pinned[reinterpret_cast<uintptr_t>(*out)] = static_cast<size_t>(bytes);
    return LP_OK;
}

void lp_host_free(void* p)
{
    if (!p)
        return;
    {
        std::lock_guard<std::mutex> lk(lprt::g_pin_mu);
        lprt::g_pinned.erase(reinterpret_cast<uintptr_t>(p));
    }
    cudaFreeHost(p);
}

lp_status lp_debug_math_sweep(lp_context* ctx, int32_t kind, uint64_t first, uint64_t count, uint64_t stats[3],
                              uint64_t* first_bad)
{
    if (!ctx || !stats || !first_bad || kind < 0 || kind > 2)
        return LP_ERR_BAD_ARG;
    LP_TRY(ensure_device(ctx));
    char* m;
    LP_TRY(poly_scratch(ctx, 1024, &m));
    unsigned long long* d = reinterpret_cast<unsigned long long*>(m);
    const unsigned long long init[4] = {0ull, 0ull, 0ull, ~0ull};
    LP_CUDA(ctx, cudaMemcpyAsync(d, init, sizeof(init), cudaMemcpyHostToDevice, ctx->stream));
    Launcher L;
    L.stream = ctx->stream;
    L.launches = &ctx->launches;
    launch_debug_math_sweep(L, kind, first, count, d, d + 3);
    if (L.err != cudaSuccess)
        return cuda_fail(ctx, L.err, "lp_debug_math_sweep launch");
    unsigned long long res[4];
    LP_CUDA(ctx, cudaMemcpyAsync(res, d, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
    LP_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int k = 0; k < 3; ++k)
        stats[k] = res[k];
    *first_bad = res[3];
    return LP_OK;
}

} // extern "C"
