// lp_io.cu — scan inputs read and results written directly in the caller's page-locked host
// buffers, over the GPU's coherent host link (NVLink-C2C on GB300), one kernel each way instead of
// one copy per array per scan. Used by lp_process_batch when every buffer of the call was
// allocated with lp_host_alloc.
#include <algorithm>

#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
// Input points (and rings) of every scan into the batch arrays. A small grid-strided grid (two
// CTAs per SM) with four host loads in flight per thread: the host link's rate needs far fewer
// threads than one per point, and the other parts of a split batch keep the remaining SMs for
// their compute while this part's inputs stream in.
__global__ void k_io_in(BatchDev b, const IoScan* io)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < b.nsrc; i0 += 4u * stride)
    {
        float4 v[4];
        uint16_t rg[4] = {0, 0, 0, 0};
        uint32_t at[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
        {
            const uint32_t i = i0 + static_cast<uint32_t>(u) * stride;
            at[u] = 0xffffffffu;
            if (i >= b.nsrc)
                continue;
            const int s = find_scan(b.nscan, i, [&](int q) { return b.scans[q].src_off; });
            const ScanDev& sd = b.scans[s];
            const uint32_t k = i - sd.src_off;
            if (k >= sd.n_src)
                continue;
            const IoScan& d = io[s];
            v[u] = reinterpret_cast<const float4*>(d.xyzi)[k];
            if (b.ring_in && d.ring)
                rg[u] = d.ring[k];
            at[u] = i;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (at[u] != 0xffffffffu)
            {
                const_cast<float4*>(b.src)[at[u]] = v[u];
                if (b.ring_in)
                    const_cast<uint16_t*>(b.ring_in)[at[u]] = rg[u];
            }
    }
}

// Per-point labels of every scan into the caller's buffers, four consecutive points per thread
// (chunk q of the batch: scan s with io[s].q_off <= q, points 4 (q - q_off) ..): the host link
// takes whole 16-byte stores (4 B of noise labels, 16 B of segmentation and of cluster labels)
// where the caller's buffers are aligned for them, and one store per label otherwise.
__device__ __forceinline__ void io_out_chunk(const BatchDev& b, const IoScan* io, uint32_t q)
{
    const int s = find_scan(b.nscan, q, [&](int t) { return io[t].q_off; });
    const ScanDev& sd = b.scans[s];
    const IoScan& d = io[s];
    const uint32_t k0 = 4u * (q - d.q_off);
    if (k0 >= sd.n_src)
        return;
    const uint32_t i0 = sd.src_off + k0;
    const uint32_t cnt = min(4u, sd.n_src - k0);
    uint8_t nz[4] = {0, 0, 0, 0};
    uint32_t sg[4] = {0, 0, 0, 0};
    int32_t cl[4] = {0, 0, 0, 0};
#pragma unroll
    for (uint32_t u = 0; u < 4; ++u)
        if (u < cnt)
        {
            // a device array is read only when the caller asked for it (stages may not produce it)
            if (d.noise)
                nz[u] = b.noise[i0 + u];
            if (d.seg)
                sg[u] = b.out_seg[i0 + u];
            if (d.cl)
                cl[u] = static_cast<int32_t>(b.out_cl[i0 + u]);
        }
    if (d.vec && cnt == 4u)
    {
        if (d.noise)
            *reinterpret_cast<uint32_t*>(d.noise + k0) =
                static_cast<uint32_t>(nz[0]) | (static_cast<uint32_t>(nz[1]) << 8) |
                (static_cast<uint32_t>(nz[2]) << 16) | (static_cast<uint32_t>(nz[3]) << 24);
        if (d.seg)
            *reinterpret_cast<uint4*>(d.seg + k0) = make_uint4(sg[0], sg[1], sg[2], sg[3]);
        if (d.cl)
            *reinterpret_cast<int4*>(d.cl + k0) = make_int4(cl[0], cl[1], cl[2], cl[3]);
        return;
    }
    for (uint32_t u = 0; u < cnt; ++u)
    {
        if (d.noise)
            d.noise[k0 + u] = nz[u];
        if (d.seg)
            d.seg[k0 + u] = sg[u];
        if (d.cl)
            d.cl[k0 + u] = cl[u];
    }
}

__global__ void k_io_out_points(BatchDev b, const IoScan* io, uint32_t nq)
{
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x)
        io_out_chunk(b, io, q);
}

// Per-cluster results: hull offsets (relative to the scan), hull indices, z range, boxes. A scan
// whose clusters or hull indices exceed the caller's capacities gets none of them (the host
// reports LP_ERR_CAPACITY for it). ret[s] = the scan's hull index count.
__global__ void k_io_out_clusters(BatchDev b, const IoScan* io, uint32_t* ret, int with_obb)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.ncl)
        return;
    const int s = find_scan(b.nscan, g, [&](int q) { return b.scans[q].cl_off; });
    const ScanDev& sd = b.scans[s];
    const uint32_t kcl = b.state[s].n_clusters;
    const uint32_t k = g - sd.cl_off;
    if (k > kcl)
        return;
    const uint32_t base = b.hull_cnt[sd.cl_off];
    const uint32_t nh = b.hull_cnt[sd.cl_off + kcl] - base;
    if (k == 0)
        ret[s] = nh;
    const IoScan& d = io[s];
    if (kcl > d.cluster_cap || nh > d.hull_cap)
        return;
    if (d.hoff)
        d.hoff[k] = b.hull_cnt[g] - base;
    if (k == kcl)
        return;
    const uint32_t h0 = b.hull_cnt[g], h1 = b.hull_cnt[g + 1];
    if (d.hidx)
        for (uint32_t j = h0; j < h1; ++j)
            d.hidx[j - base] = b.hull_out[j];
    if (d.zmin)
        d.zmin[k] = b.cl_zmin[g];
    if (d.zmax)
        d.zmax[k] = b.cl_zmax[g];
    if (with_obb)
    {
        if (d.obbc)
            d.obbc[k] = b.obb_c[g];
        if (d.obbp)
            d.obbp[k] = b.obb_p[g];
    }
}
} // namespace

void launch_io_in(Launcher& L, const BatchDev& b, const IoScan* io)
{
    LP_LAUNCH(L, k_io_in, std::min(div_up(b.nsrc, 256u), static_cast<uint32_t>(sm_count()) * 2u), 256, b, io);
}

void launch_io_out(Launcher& L, const BatchDev& b, const IoScan* io, uint32_t* ret, int with_hull, int with_obb,
                   uint32_t nq)
{
    LP_LAUNCH(L, k_io_out_points, std::min(div_up(nq, 256u), static_cast<uint32_t>(sm_count()) * 2u), 256, b, io, nq);
    if (with_hull)
        LP_LAUNCH(L, k_io_out_clusters, div_up(b.ncl, 256u), 256, b, io, ret, with_obb);
}
} // namespace lpg
