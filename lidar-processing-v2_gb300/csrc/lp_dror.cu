// lp_dror.cu — dynamic-radius outlier removal and the batch bookkeeping kernels (state
// initialisation, noise compaction, per-input-point outputs).
//
// Reference: NoiseRemover::filter, lidar_processing_lib/src/noise_remover.cpp:38-68. Per point the
// squared search radius is r2 = max(float(s2 * double(x*x + y*y)), rmin^2) with s2 =
// pow(double(multiplier), 2) (computed on the host); a point is NOISE when fewer than
// min_neighbours points, itself included, satisfy d0 + (d1 + d2) <= r2 with dk = (q_k - p_k)^2
// in binary32, query first (kdtree.hpp:131-143, :363). Counting runs over range-banded grids
// (below) so that the 27 cells around a point hold every candidate; the count stops at
// min_neighbours.
#include "lp_batch.cuh"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
constexpr unsigned long long kDEmpty = ~0ull;

__device__ __forceinline__ int scan_of_src(const BatchDev& b, uint32_t i)
{
    return find_scan(b.nscan, i, [&](int s) { return b.scans[s].src_off; });
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

__global__ void k_state_init(BatchDev b, int noise)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b.nscan)
        return;
    ScanState& st = b.state[s];
    st.n_pts = noise ? 0u : b.scans[s].n;
}

// Range bands. The radius grows with the horizontal range rho: r = rmin for rho below
// rho_c = rmin / sqrt(s2), then proportional to rho. Band 0 is [0, rho_c); band b >= 1 is
// [rho_c q^(b-1), rho_c q^b) with q = 1.25. Each band has its own grid whose cell edge bounds
// every radius in the band, and every point is also inserted into the neighbouring bands whose
// range it lies within one of their cells of, so the 27 cells around a query in its own band
// hold all its neighbours.
constexpr int kBands = 48;
constexpr float kBandQ = 1.25f;

__device__ __forceinline__ float band_rho_c(const ScanDev& sd)
{
    if (!(sd.dror_s2 > 0.0))
        return INFINITY;
    return fmaxf(static_cast<float>(sqrt(static_cast<double>(sd.dror_rmin2) / sd.dror_s2)), 1e-3f);
}

__device__ __forceinline__ int band_of(float rho, float rho_c)
{
    if (!(rho >= rho_c))
        return 0;
    const int bnd = 1 + static_cast<int>(floorf(log2f(rho / rho_c) / log2f(kBandQ)));
    return min(max(bnd, 1), kBands - 1);
}

__device__ __forceinline__ float band_cell(const ScanDev& sd, int bnd, float rho_c)
{
    double r2 = static_cast<double>(sd.dror_rmin2);
    if (bnd > 0 && isfinite(rho_c))
    {
        const double hi = static_cast<double>(rho_c) * pow(static_cast<double>(kBandQ), bnd);
        r2 = fmax(sd.dror_s2 * hi * hi, r2);
    }
    return static_cast<float>(sqrt(r2)) * 1.001f + 1e-5f;
}

__device__ __forceinline__ float horiz(const float4& p)
{
    return sqrtf(p.x * p.x + p.y * p.y);
}

__global__ void k_dror_r2(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc)
        return;
    const int s = scan_of_src(b, i);
    const ScanDev& sd = b.scans[s];
    const float4 p = b.src[i];
    // noise_remover.cpp:55-57: float products and sum, widened, scaled, narrowed, floored
    const double rho2 = static_cast<double>((p.x * p.x) + (p.y * p.y));
    b.dr2[i] = fmaxf(__double2float_rn(sd.dror_s2 * rho2), sd.dror_rmin2);
}

__device__ __forceinline__ void cell_of(const float4& p, float c, int32_t& ix, int32_t& iy, int32_t& iz)
{
    ix = static_cast<int32_t>(floorf(p.x / c));
    iy = static_cast<int32_t>(floorf(p.y / c));
    iz = static_cast<int32_t>(floorf(p.z / c));
}

__device__ __forceinline__ unsigned long long band_key(int bnd, int32_t ix, int32_t iy, int32_t iz)
{
    const unsigned long long ux = static_cast<uint32_t>(ix + (1 << 18)) & 0x7ffffu;
    const unsigned long long uy = static_cast<uint32_t>(iy + (1 << 18)) & 0x7ffffu;
    const unsigned long long uz = static_cast<uint32_t>(iz + (1 << 18)) & 0x7ffffu;
    return (static_cast<unsigned long long>(bnd) << 57) | (ux << 38) | (uy << 19) | uz;
}

// Each point goes into its own band's grid and into neighbouring bands within one cell; entry
// 3 * i + j holds the j-th insertion of point i.
__global__ void k_dror_insert(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc)
        return;
    const int s = scan_of_src(b, i);
    const ScanDev& sd = b.scans[s];
    ScanState& st = b.state[s];
    const float4 p = b.src[i];
    const float rho_c = band_rho_c(sd);
    const float rho = horiz(p);
    const int own = band_of(rho, rho_c);
    const float margin = band_cell(sd, min(own + 1, kBands - 1), rho_c) * 1.01f;
    const int lo = band_of(fmaxf(rho - margin, 0.0f), rho_c);
    const int hi = min(band_of(rho + margin, rho_c), lo + 2);
    const uint32_t mask = sd.dhash_cap - 1u;
    for (int j = 0; j < 3; ++j)
    {
        const uint32_t e = 3u * i + static_cast<uint32_t>(j);
        b.dslot[e] = 0xffffffffu;
        const int bnd = lo + j;
        if (bnd > hi)
            continue;
        int32_t ix, iy, iz;
        cell_of(p, band_cell(sd, bnd, rho_c), ix, iy, iz);
        const unsigned long long key = band_key(bnd, ix, iy, iz);
        uint32_t h = static_cast<uint32_t>(mix64(key)) & mask;
        bool placed = false;
        for (uint32_t probe = 0; probe < sd.dhash_cap; ++probe)
        {
            const uint32_t slot = sd.dhash_off + h;
            const unsigned long long prev = atomicCAS(&b.dkey[slot], kDEmpty, key);
            if (prev == kDEmpty || prev == key)
            {
                b.dslot[e] = slot;
                b.drank[e] = atomicAdd(&b.dcnt[slot], 1u);
                placed = true;
                break;
            }
            h = (h + 1u) & mask;
        }
        if (!placed)
            raise_err(&st, ERR_HASH_FULL);
    }
}

__global__ void k_dror_scatter(BatchDev b)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= 3u * b.nsrc || b.dslot[e] == 0xffffffffu)
        return;
    b.dorder[b.dstart[b.dslot[e]] + b.drank[e]] = e / 3u;
}

__device__ __forceinline__ uint32_t dlookup(const BatchDev& b, const ScanDev& sd, unsigned long long key)
{
    const uint32_t mask = sd.dhash_cap - 1u;
    uint32_t h = static_cast<uint32_t>(mix64(key)) & mask;
    for (uint32_t probe = 0; probe < sd.dhash_cap; ++probe)
    {
        const unsigned long long k = b.dkey[sd.dhash_off + h];
        if (k == key)
            return sd.dhash_off + h;
        if (k == kDEmpty)
            return 0xffffffffu;
        h = (h + 1u) & mask;
    }
    return 0xffffffffu;
}

__global__ void k_dror_query(BatchDev b)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b.nsrc)
        return;
    const int s = scan_of_src(b, i);
    const ScanDev& sd = b.scans[s];
    const float4 q = b.src[i];
    const float r2 = b.dr2[i];
    const float rho_c = band_rho_c(sd);
    const int bnd = band_of(horiz(q), rho_c);
    int32_t ix, iy, iz;
    cell_of(q, band_cell(sd, bnd, rho_c), ix, iy, iz);
    uint32_t cnt = 0;
    const uint32_t k = sd.dror_k;
    for (int dz = -1; dz <= 1 && cnt < k; ++dz)
        for (int dy = -1; dy <= 1 && cnt < k; ++dy)
            for (int dx = -1; dx <= 1 && cnt < k; ++dx)
            {
                const uint32_t slot = dlookup(b, sd, band_key(bnd, ix + dx, iy + dy, iz + dz));
                if (slot == 0xffffffffu)
                    continue;
                const uint32_t a = b.dstart[slot], e = b.dstart[slot + 1];
                for (uint32_t t = a; t < e && cnt < k; ++t)
                {
                    const float4 p = b.src[b.dorder[t]];
                    const float d0 = (q.x - p.x) * (q.x - p.x);
                    const float d1 = (q.y - p.y) * (q.y - p.y);
                    const float d2 = (q.z - p.z) * (q.z - p.z);
                    if (d0 + (d1 + d2) <= r2)
                        ++cnt;
                }
            }
    b.noise[i] = (cnt < k) ? LP_NOISE_NOISE : LP_NOISE_VALID;
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

void launch_noise(Launcher& L, const BatchDev& b, const BatchHost& hb, const lp_noise_remover_config& cfg)
{
    (void)hb;
    (void)cfg;
    const uint32_t T = 256;
    LP_LAUNCH(L, k_dror_r2, div_up(b.nsrc, T), T, b);
    LP_LAUNCH(L, k_dror_insert, div_up(b.nsrc, T), T, b);
    L.scan(b.dcnt, b.dstart, b.ndhash + 1);
    LP_LAUNCH(L, k_dror_scatter, div_up(3u * b.nsrc, T), T, b);
    LP_LAUNCH(L, k_dror_query, div_up(b.nsrc, T), T, b);
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
