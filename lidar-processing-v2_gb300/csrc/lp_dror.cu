// lp_dror.cu — batch bookkeeping around the outlier filter: state initialisation, the compaction
// of VALID points that segmentation sees (processor order: DROR first, then the VALID points in
// order), and the per-input-point outputs. The filter itself (NoiseRemover::filter,
// noise_remover.cpp:38-68) is lp_kdtree.cu.
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
__device__ __forceinline__ int scan_of_src(const BatchDev& b, uint32_t i)
{
    return find_scan(b.nscan, i, [&](int s) { return b.scans[s].src_off; });
}

__global__ void k_state_init(BatchDev b, int noise)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    ScanState& st = b.state[s];
    st.n_pts = noise ? 0u : b.scans[s].n;
}

// VALID input points are packed, in order, at the start of their scan's point slice.
__global__ void k_noise_flag(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > b.nsrc)
        return;
    b.src_pos[i] = (i < b.nsrc && b.noise[i] == LP_NOISE_VALID) ? 1u : 0u;
}

__global__ void k_noise_compact(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc || b.noise[i] != LP_NOISE_VALID)
        return;
    const int s = scan_of_src(b, i);
    const ScanDev& sd = b.scans[s];
    const uint32_t pos = sd.pt_off + (b.src_pos[i] - b.src_pos[sd.src_off]);
    b.pts[pos] = b.src[i];
    b.pt_src[pos] = static_cast<int32_t>(i);
    if (b.ring_in)
        b.ring[pos] = b.ring_in[i];
}

__global__ void k_noise_count(BatchDev b)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    const ScanDev& sd = b.scans[s];
    b.state[s].n_pts = b.src_pos[sd.src_off + sd.n_src] - b.src_pos[sd.src_off];
}

// Per input point outputs: segmentation label and cluster label (obstacle points only).
__global__ void k_outputs(BatchDev b, int with_clusters)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= b.npts)
        return;
    const int s = scan_of_point(b, j);
    if (j - b.scans[s].pt_off >= b.state[s].n_pts)
        return;
    const uint32_t src = b.pt_src ? static_cast<uint32_t>(b.pt_src[j]) : j;
    const uint32_t lbl = b.seg_label[j];
    b.out_seg[src] = lbl;
    if (with_clusters && lbl == LP_LABEL_OBSTACLE)
        b.out_cl[src] = b.obs_label[b.obs_flag[j]];
}
} // namespace

void launch_state_init(Launcher& L, const BatchDev& b, int noise)
{
    LP_LAUNCH(L, k_state_init, div_up(static_cast<uint32_t>(b.nscan), 64u), 64, b, noise);
}

void launch_noise_compaction(Launcher& L, const BatchDev& b, const BatchHost& hb)
{
    (void)hb;
    const uint32_t T = 256;
    LP_LAUNCH(L, k_noise_flag, div_up(b.nsrc + 1, T), T, b);
    L.scan(b.src_pos, b.src_pos, b.nsrc + 1);
    LP_LAUNCH(L, k_noise_compact, div_up(b.nsrc, T), T, b);
    LP_LAUNCH(L, k_noise_count, div_up(static_cast<uint32_t>(b.nscan), 64u), 64, b);
}

void launch_outputs(Launcher& L, const BatchDev& b, int with_clusters)
{
    LP_LAUNCH(L, k_outputs, div_up(b.npts, 256u), 256, b, with_clusters);
}
} // namespace lpg
