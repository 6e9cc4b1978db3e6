// lp_oracle.cpp — CPU restatement of the reference per-scan perception path.
//
// TEST INFRASTRUCTURE ONLY. This is the parity oracle: tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py call it as the checker (and as the timed CPU baseline). The GPU
// library never links, loads or calls it.
//
// Each function restates the reference algorithm (paths inside YevgeniyEngineer/LiDAR-Processing-V2)
// in the same floating-point operation order, with -ffp-contract=off so that no a*b+c is fused.
// It is pinned against the reference's own code compiled here (oracle/_ref, see build_ref.sh)
// by tests/test_oracle_pin.py on the committed fixtures in tests/golden/.
//
// libm: the reference calls glibc's atan2f/atanf/expf, which are not correctly rounded and
// differ between glibc builds (x86-64 vs aarch64 with contraction). The oracle therefore has two
// modes: LPO_LIBM_HOST calls the host libm exactly as the reference does (used to pin the
// restatement against the reference build), LPO_LIBM_CR uses correctly rounded results (the
// contract the GPU library implements). The CR values are computed in long double (x87 64-bit
// or IEEE quad significand) with an explicit rounding-ambiguity check, independently of the
// GPU's double/double-double implementation.
#include "lidar_gb300.h"

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <random>
#include <unordered_map>
#include <vector>

#include "eigen_svd2.h"
#include "introsort.h"

namespace
{
int g_libm_mode = 0;  // 0 = CR, 1 = host libm
int g_hull_ties = 0;  // 0 = equal (x, y) ordered by index, 1 = in libstdc++ std::sort's order

// convexHull's sort comparator, polygonizer.cpp:51-59 (PointXY: double, epsilon = DBL_EPSILON)
struct RefHullLess
{
    const double* xy;
    bool operator()(int32_t i, int32_t j) const
    {
        return xy[2 * i] < xy[2 * j] ||
               (std::fabs(xy[2 * i] - xy[2 * j]) < std::numeric_limits<double>::epsilon() &&
                xy[2 * i + 1] < xy[2 * j + 1]);
    }
};

constexpr float DEG_TO_RAD = static_cast<float>(M_PI / 180.0); // segmenter.hpp:135
constexpr float TWO_M_PIf = static_cast<float>(2.0 * M_PI);    // segmenter.hpp:136

// Round a long double to float, asserting the long double carried enough precision: if the
// value sits so close to a float rounding boundary that the long double error could flip it,
// fall back to the host float function's neighbour check (never observed; counted).
long g_cr_ambiguous = 0;

float roundChecked(long double v)
{
    const float f = static_cast<float>(v);
    const long double rel = (sizeof(long double) > 8) ? 1e-17L : 1e-15L;
    const float lo = static_cast<float>(v - std::fabs(v) * rel);
    const float hi = static_cast<float>(v + std::fabs(v) * rel);
    if (lo != hi)
    {
        ++g_cr_ambiguous;
    }
    return f;
}

float crAtan2f(float y, float x)
{
    return roundChecked(std::atan2(static_cast<long double>(y), static_cast<long double>(x)));
}
float crAtanf(float x)
{
    return roundChecked(std::atan(static_cast<long double>(x)));
}
float crExpf(float x)
{
    return roundChecked(std::exp(static_cast<long double>(x)));
}

inline float oAtan2f(float y, float x)
{
    return g_libm_mode ? std::atan2(y, x) : crAtan2f(y, x);
}
inline float oAtanf(float x)
{
    return g_libm_mode ? std::atan(x) : crAtanf(x);
}
inline float oExpf(float x)
{
    return g_libm_mode ? std::exp(x) : crExpf(x);
}

// common.hpp:33-62 — the reference's own minimax atan2 (no libm), same operation order.
inline float atan2Approx(float y, float x)
{
    const float ax = std::fabs(x);
    const float ay = std::fabs(y);
    const float mx = std::max(ay, ax);
    const float mn = std::min(ay, ax);
    const float a = mn / mx;
    const float s = a * a;
    const float c = s * a;
    const float q = s * s;
    float r = 0.024840285F * q + 0.18681418F;
    const float t = -0.094097948F * q - 0.33213072F;
    r = r * s + t;
    r = r * c + a;
    if (ay > ax)
        r = 1.57079637F - r;
    if (x < 0)
        r = 3.14159274F - r;
    if (y < 0)
        r = -r;
    return r;
}
} // namespace

extern "C" {

void lpo_set_libm_mode(int mode)
{
    g_libm_mode = mode;
}
// Order of hull points with the same (x, y): 1 as the reference's std::sort leaves them (libstdc++'s
// introsort restated in introsort.h, with its comparator; the GPU's order), 0 by input index (kept to
// show where the order matters).
void lpo_set_hull_ties(int mode)
{
    g_hull_ties = mode;
}
// The reference comparator's index sort four ways, for checking the restatement against the
// library: 0 restated std::sort, 1 std::sort, 2 restated with depth limit 0 (its heapsort path),
// 3 std::partial_sort(first, last, last) (libstdc++'s heapsort for that path).
int32_t lpo_debug_sort(const double* xy, uint32_t n, int variant, int32_t* out)
{
    std::iota(out, out + n, 0);
    const RefHullLess less{xy};
    if (variant == 0)
        lpo_sort::sort(out, n, less);
    else if (variant == 1)
        std::sort(out, out + n, less);
    else if (variant == 2)
        lpo_sort::sort(out, n, less, 0);
    else if (variant == 3)
        std::partial_sort(out, out + n, out + n, less);
    else
        return LP_ERR_BAD_ARG;
    return LP_OK;
}
long lpo_cr_ambiguous_count(void)
{
    return g_cr_ambiguous;
}
float lpo_math(int kind, float a, float b)
{
    switch (kind)
    {
    case 0:
        return oAtan2f(a, b);
    case 1:
        return oAtanf(a);
    case 2:
        return oExpf(a);
    default:
        return atan2Approx(a, b);
    }
}

void lpo_segmenter_config_default(lp_segmenter_config* c)
{
    // segmenter.hpp:91-108
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

// ---------------------------------------------------------------------------------------------
// Ring partition — Dataloader::addRingInfo, src/dataloader/src/dataloader.cpp:68-137.
// Quadrant of atan2 wrapped to [0, 2pi) against M_PI_2f / M_PIf / 1.5F*M_PIf (:96-114); each
// FOURTH->FIRST change decrements the ring while it is above 0 (:116-122). The start ring is a
// parameter (63 in the reference, :87).
// ---------------------------------------------------------------------------------------------
lp_status lpo_add_ring_info(const float* xyzi, uint32_t n, uint16_t first_ring, uint16_t* ring_out)
{
    int prev = 0; // FIRST
    uint16_t ring = first_ring;
    const float M_PI_2F = static_cast<float>(M_PI_2);
    const float M_PIF = static_cast<float>(M_PI);
    for (uint32_t i = 0; i < n; ++i)
    {
        float az = oAtan2f(xyzi[4 * i + 1], xyzi[4 * i + 0]);
        az = (az < 0) ? (az + 2.0F * M_PIF) : az;
        int q;
        if (az < M_PI_2F)
            q = 0;
        else if (az < M_PIF)
            q = 1;
        else if (az < 1.5F * M_PIF)
            q = 2;
        else
            q = 3;
        if (q == 0 && prev == 3 && ring > 0)
            --ring;
        prev = q;
        ring_out[i] = ring;
    }
    return LP_OK;
}

// ---------------------------------------------------------------------------------------------
// Segmentation — Segmenter::segment, lidar_processing_lib/src/segmenter.cpp:87-669.
// ---------------------------------------------------------------------------------------------
namespace
{
struct SegPoint
{
    float x, y, z;
    uint32_t label;
    uint16_t h, w;
    int32_t idx;
};

enum : uint8_t
{
    PX_EMPTY = 0,      // (0,0,0)
    PX_GROUND = 1,     // (0,255,0)
    PX_OBSTACLE = 2,   // (0,0,255)
    PX_INTER_UNK = 3,  // (0,255,255) ground pixel whose red channel was dilated
    PX_INTERSECT = 4,  // (255,0,0)
    PX_UNKNOWN = 5,    // (255,255,255)
    PX_EMPTY_RED = 6   // (0,0,255) empty pixel whose red channel was dilated
};

void pixelBGR(uint8_t s, uint8_t* out)
{
    static const uint8_t bgr[7][3] = {{0, 0, 0},     {0, 255, 0},   {0, 0, 255},  {0, 255, 255},
                                      {255, 0, 0},   {255, 255, 255}, {0, 0, 255}};
    out[0] = bgr[s][0];
    out[1] = bgr[s][1];
    out[2] = bgr[s][2];
}
} // namespace

lp_status lpo_segment(const float* xyzi, const uint16_t* ring, uint32_t n, const lp_segmenter_config* cp,
                      uint32_t* labels, uint8_t* image_out)
{
    const lp_segmenter_config& c = *cp;
    if (c.image_width <= 0 || c.image_height <= 0)
        return LP_ERR_BAD_ARG;
    // Segmenter::config, segmenter.cpp:38-71
    const float slice_res_rad = c.grid_slice_resolution_deg * DEG_TO_RAD;
    const int32_t nrad = static_cast<int32_t>(c.max_distance_m / c.grid_radial_spacing_m);
    const int32_t nslice = static_cast<int32_t>(TWO_M_PIf / slice_res_rad);
    const int32_t H = c.image_height, W = c.image_width;
    if (nrad <= 0 || nslice <= 0)
        return LP_ERR_BAD_ARG;
    std::vector<std::vector<SegPoint>> grid(static_cast<size_t>(nrad) * nslice);
    std::vector<float> elev(grid.size(), FLT_MAX);

    for (uint32_t i = 0; i < n; ++i)
        labels[i] = LP_LABEL_UNKNOWN;

    // constructPolarGrid, segmenter.cpp:103-204
    const float up = c.elevation_up_deg * DEG_TO_RAD;
    const float down = c.elevation_down_deg * DEG_TO_RAD;
    const float vfov = up - down;
    const float rad_per_px = vfov / static_cast<float>(H);
    const float zmin_adj = -c.sensor_height_m + c.z_min_m;
    const float zmax_adj = -c.sensor_height_m + c.z_max_m;
    const bool use_ring = ring != nullptr && !c.assume_unorganized_cloud;
    for (uint32_t i = 0; i < n; ++i)
    {
        const float x = xyzi[4 * i], y = xyzi[4 * i + 1], z = xyzi[4 * i + 2];
        if (z < zmin_adj || z > zmax_adj)
            continue;
        const float d = std::sqrt(x * x + y * y);
        const int32_t radial = static_cast<int32_t>(d / c.grid_radial_spacing_m);
        if (d < c.min_distance_m || d > c.max_distance_m || radial >= nrad)
            continue;
        float az = atan2Approx(y, x);
        az = (az < 0) ? (az + TWO_M_PIf) : az;
        const int32_t slice = std::min(static_cast<int32_t>(az / slice_res_rad), nslice - 1);
        uint16_t h;
        if (use_ring)
        {
            h = ring[i];
            if (h >= H)
                continue;
        }
        else
        {
            const float el = oAtanf(z / d);
            const int32_t hs = static_cast<int32_t>((el - down) / rad_per_px);
            if (hs < 0 || hs >= H)
                continue;
            h = static_cast<uint16_t>(hs);
        }
        const uint16_t w = static_cast<uint16_t>(static_cast<float>(W - 1) * az / TWO_M_PIf);
        grid[static_cast<size_t>(slice) * nrad + radial].push_back(
            {x, y, z, LP_LABEL_GROUND, h, w, static_cast<int32_t>(i)});
    }

    // RECM elevation chain, segmenter.cpp:206-267
    const float delta = std::min(c.grid_radial_spacing_m * std::tan(c.road_maximum_slope_m_per_m),
                                 c.ground_height_threshold_m - FLT_EPSILON);
    std::vector<float> zs;
    for (int32_t s = 0; s < nslice; ++s)
    {
        const size_t off = static_cast<size_t>(s) * nrad;
        elev[off] = -c.sensor_height_m + c.ground_height_threshold_m;
        float prev = elev[off];
        for (int32_t r = 1; r < nrad; ++r)
        {
            const auto& cell = grid[off + r];
            if (cell.empty())
            {
                elev[off + r] = prev + delta;
                prev = elev[off + r];
                continue;
            }
            zs.clear();
            for (const auto& p : cell)
                zs.push_back(p.z);
            std::sort(zs.begin(), zs.end());
            float zlow = zs[0];
            for (int32_t k = static_cast<int32_t>(zs.size()) / 2; k >= 1; --k)
            {
                if (zs[k] - zs[k - 1] > 0.5F)
                {
                    zlow = zs[k];
                    break;
                }
            }
            elev[off + r] = std::min(zlow, prev + delta);
            prev = elev[off + r];
        }
    }
    // classification, segmenter.cpp:269-283
    for (size_t ci = 0; ci < grid.size(); ++ci)
        for (auto& p : grid[ci])
            if (p.z >= elev[ci] + c.ground_height_threshold_m)
                p.label = LP_LABEL_OBSTACLE;

    // correctCloseRangeFalsePositivesRANSAC, segmenter.cpp:321-479
    {
        const int32_t MAX_RADIAL = 4;
        std::vector<std::array<float, 3>> rp;
        for (int32_t s = 0; s < nslice; ++s)
            for (int32_t r = 0; r < MAX_RADIAL && r < nrad; ++r)
            {
                const size_t ci = static_cast<size_t>(s) * nrad + r;
                for (const auto& p : grid[ci])
                    if (std::fabs(elev[ci] - p.z) < 2.0F * c.ground_height_threshold_m)
                        rp.push_back({p.x, p.y, p.z});
            }
        // The reference draws p3 until it differs from p2; with one candidate that never ends
        // (segmenter.cpp:382-386). Fewer than two candidates: no correction.
        if (rp.size() >= 2)
        {
            const float p1x = 0.0F, p1y = 0.0F, p1z = -c.sensor_height_m;
            const float max_cos = std::cos(std::tan(c.road_maximum_slope_m_per_m));
            float a = 0.0F, b = 0.0F, cc = 1.0F, dd = 0.0F;
            std::mt19937 gen{42};
            std::uniform_int_distribution<uint32_t> dist{0, static_cast<uint32_t>(rp.size()) - 1U};
            uint32_t best = 0;
            for (uint32_t it = 0; it < 60; ++it)
            {
                const uint32_t i2 = dist(gen);
                uint32_t i3 = dist(gen);
                while (i3 == i2)
                    i3 = dist(gen);
                const auto& p2 = rp[i2];
                const auto& p3 = rp[i3];
                float nx = ((p2[1] - p1y) * (p3[2] - p1z)) - ((p2[2] - p1z) * (p3[1] - p1y));
                float ny = ((p2[2] - p1z) * (p3[0] - p1x)) - ((p2[0] - p1x) * (p3[2] - p1z));
                float nz = ((p2[0] - p1x) * (p3[1] - p1y)) - ((p2[1] - p1y) * (p3[0] - p1x));
                const float den = (nx * nx) + (ny * ny) + (nz * nz);
                if (den < 1.0e-5F)
                    continue;
                const float norm = 1.0F / std::sqrt(den);
                nz *= norm;
                if (std::fabs(nz) < max_cos)
                    continue;
                nx *= norm;
                ny *= norm;
                const float pd = (nx * p1x) + (ny * p1y) + (nz * p1z);
                uint32_t cnt = 0;
                for (const auto& p : rp)
                    if (std::fabs((nx * p[0]) + (ny * p[1]) + (nz * p[2]) - pd) < c.ground_height_threshold_m)
                        ++cnt;
                if (cnt > best)
                {
                    best = cnt;
                    a = nx;
                    b = ny;
                    cc = nz;
                    dd = pd;
                }
            }
            if (best > 0)
            {
                if (cc < 0)
                {
                    a = -a;
                    b = -b;
                    cc = -cc;
                    dd = -dd;
                }
                for (int32_t s = 0; s < nslice; ++s)
                    for (int32_t r = 0; r < MAX_RADIAL && r < nrad; ++r)
                        for (auto& p : grid[static_cast<size_t>(s) * nrad + r])
                            if ((a * p.x) + (b * p.y) + (cc * p.z) - dd < c.ground_height_threshold_m)
                                p.label = LP_LABEL_GROUND;
            }
        }
    }

    // Polar grid -> range image: nearest point per pixel wins, strict '<' (segmenter.cpp:291-318)
    const size_t npx = static_cast<size_t>(H) * W;
    std::vector<float> depth(npx, FLT_MAX);
    std::vector<int32_t> map(npx, -1);
    std::vector<uint8_t> px(npx, PX_EMPTY);
    for (const auto& cell : grid)
        for (const auto& p : cell)
        {
            const size_t ii = static_cast<size_t>(p.h) * W + p.w;
            const float d2 = (p.x * p.x) + (p.y * p.y);
            if (d2 < depth[ii])
            {
                px[ii] = (p.label == LP_LABEL_GROUND) ? PX_GROUND : PX_OBSTACLE;
                depth[ii] = d2;
                map[ii] = p.idx;
            }
        }

    // JCP, segmenter.cpp:481-638. Red-channel 5x5 dilation clipped at the image border
    // (cv::dilate default border), then the row-major intersection queue.
    std::vector<uint8_t> red(npx);
    for (size_t i = 0; i < npx; ++i)
        red[i] = (px[i] == PX_OBSTACLE) ? 1 : 0;
    std::vector<int32_t> queue;
    for (int32_t h = 0; h < H; ++h)
        for (int32_t w = 0; w < W; ++w)
        {
            bool dil = false;
            for (int32_t dh = -2; dh <= 2 && !dil; ++dh)
                for (int32_t dw = -2; dw <= 2; ++dw)
                {
                    const int32_t hh = h + dh, ww = w + dw;
                    if (hh >= 0 && hh < H && ww >= 0 && ww < W && red[static_cast<size_t>(hh) * W + ww])
                    {
                        dil = true;
                        break;
                    }
                }
            const size_t ii = static_cast<size_t>(h) * W + w;
            if (!dil)
                continue;
            if (px[ii] == PX_GROUND)
                px[ii] = PX_INTER_UNK;
            else if (px[ii] == PX_EMPTY)
                px[ii] = PX_EMPTY_RED;
            if (px[ii] == PX_INTER_UNK)
            {
                if (map[ii] != -1)
                {
                    queue.push_back(static_cast<int32_t>(ii));
                    px[ii] = PX_INTERSECT;
                }
                else
                {
                    px[ii] = PX_UNKNOWN;
                }
            }
        }
    static const int32_t off[24][2] = {{-2, -2}, {-2, -1}, {-2, 0}, {-2, 1}, {-2, 2}, {-1, -2},
                                       {-1, -1}, {-1, 0},  {-1, 1}, {-1, 2}, {0, -2}, {0, -1},
                                       {0, 1},   {0, 2},   {1, -2}, {1, -1}, {1, 0},  {1, 1},
                                       {1, 2},   {2, -2},  {2, -1}, {2, 0},  {2, 1},  {2, 2}};
    // Per-slot weights and labels persist across queue elements: a slot that falls outside the
    // image keeps the previous element's value (segmenter.cpp:523-525, :552-556).
    float wu[24];
    uint32_t lab[24];
    for (int k = 0; k < 24; ++k)
    {
        wu[k] = 0.0F;
        lab[k] = LP_LABEL_UNKNOWN;
    }
    const float kthr2 = c.kernel_threshold_distance_m * c.kernel_threshold_distance_m;
    for (int32_t ii : queue)
    {
        const int32_t h = ii / W, w = ii % W;
        const int32_t pi = map[ii];
        const float cx = xyzi[4 * pi], cy = xyzi[4 * pi + 1], cz = xyzi[4 * pi + 2];
        float sum = 0.0F;
        for (int k = 0; k < 24; ++k)
        {
            const int32_t hh = h + off[k][0], ww = w + off[k][1];
            if (hh < 0 || hh >= H || ww < 0 || ww >= W)
                continue;
            const size_t ni = static_cast<size_t>(hh) * W + ww;
            const int32_t np = map[ni];
            if (np == -1)
            {
                wu[k] = 0.0F;
                lab[k] = LP_LABEL_UNKNOWN;
                continue;
            }
            const float dx = cx - xyzi[4 * np], dy = cy - xyzi[4 * np + 1], dz = cz - xyzi[4 * np + 2];
            const float d2 = dx * dx + dy * dy + dz * dz;
            if (d2 > kthr2)
            {
                wu[k] = 0.0F;
                lab[k] = LP_LABEL_UNKNOWN;
                continue;
            }
            const float dist = std::sqrt(d2);
            wu[k] = oExpf(-c.amplification_factor * dist);
            sum += wu[k];
            lab[k] = (px[ni] == PX_GROUND) ? LP_LABEL_GROUND
                     : (px[ni] == PX_OBSTACLE) ? LP_LABEL_OBSTACLE
                                               : LP_LABEL_UNKNOWN;
        }
        if (std::fabs(sum) > FLT_EPSILON)
        {
            float wo = 0.0F, wg = 0.0F;
            for (int k = 0; k < 24; ++k)
            {
                const float wn = wu[k] / sum;
                if (lab[k] == LP_LABEL_GROUND)
                    wg += wn;
                else if (lab[k] == LP_LABEL_OBSTACLE)
                    wo += wn;
            }
            px[ii] = (wo > wg) ? PX_OBSTACLE : PX_GROUND;
        }
    }

    // populateLabels, segmenter.cpp:640-669
    for (size_t ii = 0; ii < npx; ++ii)
    {
        if (map[ii] == -1)
            continue;
        if (px[ii] == PX_GROUND)
            labels[map[ii]] = LP_LABEL_GROUND;
        else if (px[ii] == PX_OBSTACLE)
            labels[map[ii]] = LP_LABEL_OBSTACLE;
    }
    if (image_out)
        for (size_t ii = 0; ii < npx; ++ii)
            pixelBGR(px[ii], image_out + 3 * ii);
    return LP_OK;
}

// ---------------------------------------------------------------------------------------------
// DROR — NoiseRemover::filter, lidar_processing_lib/src/noise_remover.cpp:38-68.
// Radius per point: s2 = pow(double(mult), 2); rho2 = double(x*x + y*y) (float products and sum);
// r2 = max(float(s2 * rho2), rmin*rmin). Neighbour test: d0 + (d1 + d2) <= r2 with dk = (q_k -
// p_k)^2 in float, query first (kdtree.hpp:131-143, :363).
//
// mode 0 (exact): NOISE iff fewer than min_neighbours points (itself included) lie within r2.
// mode 1 (reference kd-tree): the reference's kd-tree (nth_element median split on depth % 3,
//   kdtree.hpp:161-214) and radius_search_k_nearest (kdtree.hpp:339-397), including the
//   traversal stack that is never cleared after an early break, so later queries continue
//   through subtrees left by earlier ones and may count a point more than once. The stack
//   starts empty for every call.
// ---------------------------------------------------------------------------------------------
namespace
{
inline float drorDist(const float* q, const float* p)
{
    const float d0 = (q[0] - p[0]) * (q[0] - p[0]);
    const float d1 = (q[1] - p[1]) * (q[1] - p[1]);
    const float d2 = (q[2] - p[2]) * (q[2] - p[2]);
    return d0 + (d1 + d2);
}

inline float drorRadius2(const float* p, double s2, float rmin2)
{
    // (point[0] * point[0]) + (point[1] * point[1]) is a float sum, then widened (noise_remover.cpp:55)
    const double rho2 = static_cast<double>((p[0] * p[0]) + (p[1] * p[1]));
    return std::max(static_cast<float>(s2 * rho2), rmin2);
}
} // namespace

// KDTree::rebuild (kdtree.hpp:161-214): nodes_ holds the points in input order; a stack of
// (begin, end, parent link, depth) ranges, each put in order around its middle position by
// std::nth_element on the depth's axis (x, y, z in turn), the middle becoming the node and the two
// sides its subtrees. Returns the root position; node positions are the array's.
struct KdNode
{
    float p[3];
    uint32_t index;
    int32_t left, right;
};

int32_t kdBuild(const float* P, uint32_t n, std::vector<KdNode>& nodes)
{
    nodes.resize(n);
    for (uint32_t i = 0; i < n; ++i)
        nodes[i] = {{P[3 * i], P[3 * i + 1], P[3 * i + 2]}, i, -1, -1};
    struct Build
    {
        uint32_t b, e;
        int32_t parent; // -1 root
        int side;       // 0 left, 1 right
        uint32_t depth;
    };
    int32_t root = -1;
    std::vector<Build> bs;
    bs.push_back({0, n, -1, 0, 0});
    while (!bs.empty())
    {
        const Build t = bs.back();
        bs.pop_back();
        if (t.b >= t.e)
            continue;
        const uint32_t axis = t.depth % 3;
        const uint32_t mid = t.b + (t.e - t.b) / 2;
        std::nth_element(nodes.begin() + t.b, nodes.begin() + mid, nodes.begin() + t.e,
                         [axis](const KdNode& x, const KdNode& y) { return x.p[axis] < y.p[axis]; });
        if (t.parent < 0)
            root = static_cast<int32_t>(mid);
        else if (t.side == 0)
            nodes[t.parent].left = static_cast<int32_t>(mid);
        else
            nodes[t.parent].right = static_cast<int32_t>(mid);
        if (mid > t.b)
            bs.push_back({t.b, mid, static_cast<int32_t>(mid), 0, t.depth + 1});
        if (mid + 1 < t.e)
            bs.push_back({mid + 1, t.e, static_cast<int32_t>(mid), 1, t.depth + 1});
    }
    return root;
}

// The kd-tree's points by node position (n x 3 floats), for checking a tree built elsewhere.
int32_t lpo_kdtree_positions(const float* xyz, uint32_t n, float* out_xyz)
{
    std::vector<KdNode> nodes;
    kdBuild(xyz, n, nodes);
    for (uint32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d)
            out_xyz[3 * i + d] = nodes[i].p[d];
    return 0;
}

// std::nth_element (host library) or its restatement (lpo_sort::nth_element) on float keys:
// the resulting order of the input indices. depth_override >= 0 forces the restatement's depth
// limit (0: heap selection at once).
int32_t lpo_debug_nth(const float* v, uint32_t n, uint32_t nth, int32_t restated, int32_t depth_override,
                      int32_t* order_out)
{
    struct Key
    {
        float v;
        int32_t i;
    };
    std::vector<Key> a(n);
    for (uint32_t i = 0; i < n; ++i)
        a[i] = {v[i], static_cast<int32_t>(i)};
    auto less = [](const Key& x, const Key& y) { return x.v < y.v; };
    if (restated)
        lpo_sort::nth_element(a.data(), n, nth, less, depth_override);
    else
        std::nth_element(a.begin(), a.begin() + nth, a.end(), less);
    for (uint32_t i = 0; i < n; ++i)
        order_out[i] = a[i].i;
    return 0;
}

lp_status lpo_noise_remove(const float* xyz, uint32_t stride, uint32_t n,
                           const lp_noise_remover_config* cfg, int mode, uint8_t* out)
{
    const double s2 = std::pow(static_cast<double>(cfg->radius_multiplier_m_per_m), 2.0);
    const float rmin2 = cfg->min_search_radius_m * cfg->min_search_radius_m;
    const uint32_t k = cfg->min_neighbours;
    std::vector<float> P(static_cast<size_t>(n) * 3);
    for (uint32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d)
            P[3 * i + d] = xyz[static_cast<size_t>(stride) * i + d];
    for (uint32_t i = 0; i < n; ++i)
        out[i] = LP_NOISE_VALID;
    if (n == 0)
        return LP_OK;
    if (mode == 0)
    {
        // uniform grid with cells no smaller than the largest radius
        float rmax2 = 0;
        for (uint32_t i = 0; i < n; ++i)
            rmax2 = std::max(rmax2, drorRadius2(&P[3 * i], s2, rmin2));
        const double cell = std::max(std::sqrt(static_cast<double>(rmax2)) * 1.0001, 1e-3);
        std::unordered_map<int64_t, std::vector<uint32_t>> bins;
        auto key = [&](long a, long b, long c2) { return (a * 2000003LL + b) * 2000003LL + c2; };
        std::vector<long> ci(static_cast<size_t>(n) * 3);
        for (uint32_t i = 0; i < n; ++i)
        {
            for (int d = 0; d < 3; ++d)
                ci[3 * i + d] = static_cast<long>(std::floor(P[3 * i + d] / cell));
            bins[key(ci[3 * i], ci[3 * i + 1], ci[3 * i + 2])].push_back(i);
        }
        for (uint32_t i = 0; i < n; ++i)
        {
            const float r2 = drorRadius2(&P[3 * i], s2, rmin2);
            uint32_t cnt = 0;
            for (int a = -1; a <= 1 && cnt < k; ++a)
                for (int b = -1; b <= 1 && cnt < k; ++b)
                    for (int c2 = -1; c2 <= 1 && cnt < k; ++c2)
                    {
                        auto it = bins.find(key(ci[3 * i] + a, ci[3 * i + 1] + b, ci[3 * i + 2] + c2));
                        if (it == bins.end())
                            continue;
                        for (uint32_t j : it->second)
                            if (drorDist(&P[3 * i], &P[3 * j]) <= r2 && ++cnt >= k)
                                break;
                    }
            if (cnt < k)
                out[i] = LP_NOISE_NOISE;
        }
        return LP_OK;
    }
    // mode 1: reference kd-tree with the persistent traversal stack
    std::vector<KdNode> nodes;
    const int32_t root = kdBuild(P.data(), n, nodes);
    struct Entry
    {
        int32_t node;
        uint32_t axis;
    };
    std::vector<Entry> stack;
    for (uint32_t i = 0; i < n; ++i)
    {
        const float* q = &P[3 * i];
        const float r2 = drorRadius2(q, s2, rmin2);
        uint32_t found = 0;
        stack.push_back({root, 0});
        while (!stack.empty())
        {
            const Entry e = stack.back();
            stack.pop_back();
            if (e.node < 0)
                continue;
            const KdNode& nd = nodes[e.node];
            if (drorDist(q, nd.p) <= r2)
            {
                if (++found >= k)
                    break;
            }
            const uint32_t nx = (e.axis + 1U) % 3;
            const float delta = nd.p[e.axis] - q[e.axis];
            if (delta * delta <= r2)
            {
                stack.push_back({nd.right, nx});
                stack.push_back({nd.left, nx});
            }
            else
            {
                stack.push_back({(delta > 0) ? nd.left : nd.right, nx});
            }
        }
        if (found < k)
            out[i] = LP_NOISE_NOISE;
    }
    return LP_OK;
}

// ---------------------------------------------------------------------------------------------
// Clustering — Clusterer::cluster, lidar_processing_lib/src/clusterer.cpp:43-239.
// ---------------------------------------------------------------------------------------------
lp_status lpo_cluster(const float* xyz, uint32_t stride, uint32_t n, const lp_clusterer_config* cfg,
                      int32_t* labels)
{
    if (n == 0)
        return LP_OK;
    const float res_r = cfg->voxel_grid_range_resolution_m;
    const float res_a = cfg->voxel_grid_azimuth_resolution_deg * DEG_TO_RAD;
    const float res_e = cfg->voxel_grid_elevation_resolution_deg * DEG_TO_RAD;
    // cartesianToSpherical, clusterer.cpp:55-100
    std::vector<float> R(n), A(n), E(n);
    float max_r = std::numeric_limits<float>::lowest();
    float max_a = max_r, max_e = max_r;
    const float M_PI_2F = static_cast<float>(M_PI_2);
    for (uint32_t i = 0; i < n; ++i)
    {
        const float x = xyz[static_cast<size_t>(stride) * i], y = xyz[static_cast<size_t>(stride) * i + 1],
                    z = xyz[static_cast<size_t>(stride) * i + 2];
        float az = oAtan2f(y, x);
        az = (az < 0) ? (az + TWO_M_PIf) : az;
        max_a = std::max(max_a, az);
        const float d2 = x * x + y * y;
        const float d = std::sqrt(d2);
        const float r = std::sqrt(d2 + z * z);
        max_r = std::max(max_r, r);
        const float el = oAtanf(z / d) + M_PI_2F;
        max_e = std::max(max_e, el);
        R[i] = r;
        A[i] = az;
        E[i] = el;
    }
    const int32_t nr = static_cast<int32_t>(std::ceil(max_r / res_r) + 1);
    const int32_t na = static_cast<int32_t>(std::ceil(max_a / res_a) + 1);
    const int32_t ne = static_cast<int32_t>(std::ceil(max_e / res_e) + 1);
    // buildHashTable, clusterer.cpp:102-120 (capacity 200,000 voxels, clusterer.cpp:36)
    std::vector<int32_t> vr(n), va(n), ve(n), vflat(n);
    std::unordered_map<int32_t, int32_t> vlabel;
    vlabel.reserve(1 << 18);
    for (uint32_t i = 0; i < n; ++i)
    {
        vr[i] = static_cast<int32_t>(R[i] / res_r);
        va[i] = static_cast<int32_t>(A[i] / res_a);
        ve[i] = static_cast<int32_t>(E[i] / res_e);
        vflat[i] = nr * (na * ve[i] + va[i]) + vr[i];
        vlabel.emplace(vflat[i], -1);
        if (vlabel.size() > 200000)
            return LP_ERR_CAPACITY;
    }
    // clusterImpl BFS, clusterer.cpp:122-193 (offsets table clusterer.hpp:101-105)
    int32_t label = 0;
    std::vector<std::array<int32_t, 3>> q;
    for (uint32_t i = 0; i < n; ++i)
    {
        if (vlabel[vflat[i]] != -1)
            continue;
        q.clear();
        q.push_back({vr[i], va[i], ve[i]});
        vlabel[vflat[i]] = label;
        for (size_t h = 0; h < q.size(); ++h)
        {
            const auto cur = q[h];
            for (int de = -1; de <= 1; ++de)
                for (int da = -1; da <= 1; ++da)
                    for (int dr = -1; dr <= 1; ++dr)
                    {
                        if (!dr && !da && !de)
                            continue;
                        const int32_t rr = cur[0] + dr, ee = cur[2] + de;
                        if (rr < 0 || rr >= nr || ee < 0 || ee >= ne)
                            continue;
                        int32_t aa = cur[1] + da;
                        if (aa < 0)
                            aa += na;
                        else if (aa >= na)
                            aa -= na;
                        const int32_t f = nr * (na * ee + aa) + rr;
                        auto it = vlabel.find(f);
                        if (it != vlabel.end() && it->second == -1)
                        {
                            it->second = label;
                            q.push_back({rr, aa, ee});
                        }
                    }
        }
        ++label;
    }
    for (uint32_t i = 0; i < n; ++i)
        labels[i] = vlabel[vflat[i]];
    // removeSmallClusters, clusterer.cpp:195-239
    std::vector<uint32_t> cnt(label, 0);
    for (uint32_t i = 0; i < n; ++i)
        ++cnt[labels[i]];
    std::vector<int32_t> remap(label, -1);
    int32_t cur = 0;
    for (int32_t l = 0; l < label; ++l)
        if (cnt[l] >= cfg->min_cluster_size)
            remap[l] = cur++;
    for (uint32_t i = 0; i < n; ++i)
        labels[i] = remap[labels[i]];
    return LP_OK;
}

// ---------------------------------------------------------------------------------------------
// Polygonizer — lidar_processing_lib/src/polygonizer.cpp.
// ---------------------------------------------------------------------------------------------

// convexHull, polygonizer.cpp:33-91. Sort key: (x, y); points with identical (x, y) are ordered
// by index (the reference's std::sort leaves their order to the sort implementation), or, with
// lpo_set_hull_ties(1), exactly as libstdc++'s std::sort leaves them.
lp_status lpo_convex_hull(const double* xy, uint32_t n, int32_t* out, uint32_t* n_out)
{
    if (n < 3)
    {
        for (uint32_t i = 0; i < n; ++i)
            out[i] = static_cast<int32_t>(i);
        *n_out = n;
        return LP_OK;
    }
    std::vector<int32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    if (g_hull_ties == 1)
        lpo_sort::sort(idx.data(), n, RefHullLess{xy});
    else
        std::sort(idx.begin(), idx.end(), [xy](int32_t i, int32_t j) {
            if (xy[2 * i] != xy[2 * j])
                return xy[2 * i] < xy[2 * j];
            if (xy[2 * i + 1] != xy[2 * j + 1])
                return xy[2 * i + 1] < xy[2 * j + 1];
            return i < j;
        });
    auto ccwOrColinear = [xy](int32_t a, int32_t b, int32_t c) {
        return (xy[2 * b] - xy[2 * a]) * (xy[2 * c + 1] - xy[2 * a + 1]) -
                   (xy[2 * b + 1] - xy[2 * a + 1]) * (xy[2 * c] - xy[2 * a]) <=
               0;
    };
    std::vector<int32_t> h(2 * static_cast<size_t>(n));
    int32_t k = 0;
    for (uint32_t i = 0; i < n; ++i)
    {
        while (k > 1 && ccwOrColinear(h[k - 2], h[k - 1], idx[i]))
            --k;
        h[k++] = idx[i];
    }
    for (int32_t i = static_cast<int32_t>(n) - 2, t = k + 1; i >= 0; --i)
    {
        while (k >= t && ccwOrColinear(h[k - 2], h[k - 1], idx[i]))
            --k;
        h[k++] = idx[i];
    }
    for (int32_t i = 0; i < k - 1; ++i)
        out[i] = h[i];
    *n_out = static_cast<uint32_t>(k - 1);
    return LP_OK;
}

namespace
{
// areaOfTriangle, polygonizer.hpp:227-231
inline double triArea(const double* a, const double* b, const double* c)
{
    return std::fabs((a[0] * (b[1] - c[1]) + b[0] * (c[1] - a[1]) + c[0] * (a[1] - b[1])) * 0.5);
}

// findAntipodalPairsOfConvexHull, polygonizer.cpp:93-163
void antipodal(const double* P, int32_t n, std::vector<std::array<int32_t, 2>>& pairs)
{
    pairs.clear();
    if (n < 2)
        return;
    auto nx = [n](int32_t i) { return (i + 1 == n) ? 0 : i + 1; };
    auto pt = [P](int32_t i) { return P + 2 * i; };
    const int32_t i0 = n - 1;
    int32_t i = 0, j = 1;
    while (triArea(pt(i), pt(nx(i)), pt(nx(j))) > triArea(pt(i), pt(nx(i)), pt(j)))
        j = nx(j);
    const int32_t j0 = j;
    while (i != j0)
    {
        i = nx(i);
        pairs.push_back({i, j});
        while (triArea(pt(i), pt(nx(i)), pt(nx(j))) > triArea(pt(i), pt(nx(i)), pt(j)))
        {
            j = nx(j);
            if (!(i == j0 && j == i0))
                pairs.push_back({i, j});
            else
                return;
        }
        if (triArea(pt(j), pt(nx(i)), pt(nx(j))) == triArea(pt(i), pt(nx(i)), pt(j)))
        {
            if (!(i == j0 && j == i0))
                pairs.push_back({i, nx(j)});
            else
                pairs.push_back({nx(i), j});
        }
    }
}
} // namespace

lp_status lpo_antipodal_pairs(const double* P, uint32_t n, int32_t* out, uint32_t cap, uint32_t* npairs)
{
    std::vector<std::array<int32_t, 2>> pairs;
    antipodal(P, static_cast<int32_t>(n), pairs);
    *npairs = static_cast<uint32_t>(pairs.size());
    if (pairs.size() > cap)
        return LP_ERR_CAPACITY;
    for (size_t i = 0; i < pairs.size(); ++i)
    {
        out[2 * i] = pairs[i][0];
        out[2 * i + 1] = pairs[i][1];
    }
    return LP_OK;
}

// boundingBoxRotatingCalipers, polygonizer.cpp:165-278. The running best area is stored in
// BoundingBox::area, a float (polygonizer.hpp:78): DBL_MAX converts to +inf, and each
// comparison is against the float-rounded best so far.
lp_status lpo_bounding_box_rotating_calipers(const double* P, uint32_t nu, lp_bounding_box* box)
{
    std::memset(box, 0, sizeof(*box));
    const int32_t n = static_cast<int32_t>(nu);
    if (n < 3)
        return LP_OK;
    std::vector<std::array<int32_t, 2>> pairs;
    antipodal(P, n, pairs);
    double cx = 0.0, cy = 0.0;
    for (int32_t i = 0; i < n; ++i)
    {
        cx += P[2 * i];
        cy += P[2 * i + 1];
    }
    cx /= n;
    cy /= n;
    float best = static_cast<float>(std::numeric_limits<double>::max());
    for (const auto& pr : pairs)
        for (int e = 0; e < 2; ++e)
        {
            const int32_t index = pr[e];
            for (int o = 0; o < 2; ++o)
            {
                int32_t nb = index + (o == 0 ? -1 : 1);
                if (nb < 0)
                    nb += n;
                else if (nb >= n)
                    nb -= n;
                const double ex = P[2 * nb] - P[2 * index];
                const double ey = P[2 * nb + 1] - P[2 * index + 1];
                const double len = std::sqrt(ex * ex + ey * ey);
                if (len < 1.0e-6)
                    continue;
                const double ux = ex / len, uy = ey / len;
                double mnx = std::numeric_limits<double>::max(), mxx = std::numeric_limits<double>::lowest();
                double mny = mnx, mxy = mxx;
                for (int32_t k = 0; k < n; ++k)
                {
                    const double tx = P[2 * k] - cx, ty = P[2 * k + 1] - cy;
                    const double rx = tx * ux + ty * uy;
                    const double ry = -tx * uy + ty * ux;
                    mnx = std::min(mnx, rx);
                    mxx = std::max(mxx, rx);
                    mny = std::min(mny, ry);
                    mxy = std::max(mxy, ry);
                }
                const double area = (mxx - mnx) * (mxy - mny);
                if (area < best)
                {
                    best = static_cast<float>(area);
                    box->area = best;
                    box->corners[0][0] = mnx * ux - mny * uy + cx;
                    box->corners[0][1] = mnx * uy + mny * ux + cy;
                    box->corners[1][0] = mxx * ux - mny * uy + cx;
                    box->corners[1][1] = mxx * uy + mny * ux + cy;
                    box->corners[2][0] = mxx * ux - mxy * uy + cx;
                    box->corners[2][1] = mxx * uy + mxy * ux + cy;
                    box->corners[3][0] = mnx * ux - mxy * uy + cx;
                    box->corners[3][1] = mnx * uy + mxy * ux + cy;
                    box->angle_rad = atan2Approx(static_cast<float>(uy), static_cast<float>(ux));
                    box->is_valid = 1;
                }
            }
        }
    return LP_OK;
}

// V of Eigen's JacobiSVD of a 2x2 matrix (row-major a[4] -> v[4]), for the oracle's own tests.
extern "C" int32_t lpo_jacobi_svd2(const double* a, double* v)
{
    return eigen_svd2::jacobi_svd2_v(a[0], a[1], a[2], a[3], v) ? 0 : 1;
}

// boundingBoxPrincipalComponentAnalysis, polygonizer.cpp:280-362, in FP64: mean, centred
// X^T X / (n - 1) (:321-322), V of Eigen's JacobiSVD of that covariance (:325-331, restated in
// eigen_svd2.h), rotate (:334), min/max (:337-340), corners back (:343-347).
lp_status lpo_bounding_box_pca(const double* P, uint32_t n, lp_bounding_box* box, double* cov_out)
{
    std::memset(box, 0, sizeof(*box));
    if (n < 3)
        return LP_OK;
    double mx = 0.0, my = 0.0;
    for (uint32_t i = 0; i < n; ++i)
    {
        mx += P[2 * i];
        my += P[2 * i + 1];
    }
    mx /= n;
    my /= n;
    double sxx = 0.0, sxy = 0.0, syy = 0.0;
    for (uint32_t i = 0; i < n; ++i)
    {
        const double dx = P[2 * i] - mx, dy = P[2 * i + 1] - my;
        sxx += dx * dx;
        sxy += dx * dy;
        syy += dy * dy;
    }
    sxx /= (n - 1);
    sxy /= (n - 1);
    syy /= (n - 1);
    if (cov_out)
    {
        cov_out[0] = sxx;
        cov_out[1] = sxy;
        cov_out[2] = syy;
    }
    // principal components of [[sxx, sxy], [sxy, syy]]: V of the JacobiSVD (an invalid SVD, on a
    // non-finite covariance, leaves the box invalid as at :326-330)
    double V[4];
    if (!eigen_svd2::jacobi_svd2_v(sxx, sxy, sxy, syy, V))
        return LP_OK;
    const double v00 = V[0], v01 = V[1], v10 = V[2], v11 = V[3];
    double mnx = std::numeric_limits<double>::max(), mxx = std::numeric_limits<double>::lowest();
    double mny = mnx, mxy = mxx;
    for (uint32_t i = 0; i < n; ++i)
    {
        const double dx = P[2 * i] - mx, dy = P[2 * i + 1] - my;
        const double rx = dx * v00 + dy * v10;
        const double ry = dx * v01 + dy * v11;
        mnx = std::min(mnx, rx);
        mxx = std::max(mxx, rx);
        mny = std::min(mny, ry);
        mxy = std::max(mxy, ry);
    }
    const double cxs[4] = {mnx, mxx, mxx, mnx};
    const double cys[4] = {mny, mny, mxy, mxy};
    for (int k = 0; k < 4; ++k)
    {
        box->corners[k][0] = cxs[k] * v00 + cys[k] * v01 + mx;
        box->corners[k][1] = cxs[k] * v10 + cys[k] * v11 + my;
    }
    box->area = static_cast<float>((mxx - mnx) * (mxy - mny));
    box->angle_rad = static_cast<float>(std::atan2(v10, v00));
    box->is_valid = 1;
    return LP_OK;
}

// ---------------------------------------------------------------------------------------------
// Whole scan — Processor::run, src/processor/src/processor.cpp:552-671, with optional DROR on
// the input cloud first (members declared at processor.hpp:243-246).
// ---------------------------------------------------------------------------------------------
lp_status lpo_process_scan(const lp_pipeline_config* cfg, const lp_scan_input* scan, int dror_mode,
                           lp_scan_output* out)
{
    const uint32_t n = scan->n;
    std::vector<uint8_t> noise(n, LP_NOISE_VALID);
    if (cfg->enable_noise_removal)
        lpo_noise_remove(scan->xyzi, 4, n, &cfg->noise, dror_mode, noise.data());
    std::vector<uint32_t> keep;
    for (uint32_t i = 0; i < n; ++i)
        if (noise[i] == LP_NOISE_VALID)
            keep.push_back(i);
    const uint32_t m = static_cast<uint32_t>(keep.size());
    std::vector<float> xyzi(static_cast<size_t>(m) * 4);
    std::vector<uint16_t> ring;
    for (uint32_t j = 0; j < m; ++j)
        std::memcpy(&xyzi[4 * j], &scan->xyzi[4 * static_cast<size_t>(keep[j])], 16);
    const uint16_t* ringp = nullptr;
    if (cfg->compute_ring)
    {
        ring.resize(m);
        lpo_add_ring_info(xyzi.data(), m, cfg->first_ring, ring.data());
        ringp = ring.data();
    }
    else if (scan->ring)
    {
        ring.resize(m);
        for (uint32_t j = 0; j < m; ++j)
            ring[j] = scan->ring[keep[j]];
        ringp = ring.data();
    }
    std::vector<uint32_t> seg(m);
    lp_status st = lpo_segment(xyzi.data(), ringp, m, &scan->seg, seg.data(), nullptr);
    if (st != LP_OK)
        return st;
    std::vector<uint32_t> obstacle;
    std::vector<float> obs;
    for (uint32_t j = 0; j < m; ++j)
        if (seg[j] == LP_LABEL_OBSTACLE)
        {
            obstacle.push_back(keep[j]);
            obs.insert(obs.end(), {xyzi[4 * j], xyzi[4 * j + 1], xyzi[4 * j + 2]});
        }
    const uint32_t nobs = static_cast<uint32_t>(obstacle.size());
    std::vector<int32_t> cl(nobs);
    if (nobs)
    {
        st = lpo_cluster(obs.data(), 3, nobs, &cfg->cluster, cl.data());
        if (st != LP_OK)
            return st;
    }
    if (out->noise_labels)
        std::memcpy(out->noise_labels, noise.data(), n);
    if (out->seg_labels)
    {
        std::fill(out->seg_labels, out->seg_labels + n, static_cast<uint32_t>(LP_LABEL_UNKNOWN));
        for (uint32_t j = 0; j < m; ++j)
            out->seg_labels[keep[j]] = seg[j];
    }
    if (out->cluster_labels)
    {
        std::fill(out->cluster_labels, out->cluster_labels + n, LP_INVALID_CLUSTER);
        for (uint32_t j = 0; j < nobs; ++j)
            out->cluster_labels[obstacle[j]] = cl[j];
    }
    int32_t maxl = -1;
    for (int32_t l : cl)
        maxl = std::max(maxl, l);
    const uint32_t K = static_cast<uint32_t>(maxl + 1);
    out->n_obstacles = nobs;
    out->n_clusters = K;
    if (K > out->cluster_capacity)
        return LP_ERR_CAPACITY;
    // gather per cluster in obstacle order (processor.cpp:627-658), then hull + boxes
    std::vector<std::vector<uint32_t>> members(K);
    for (uint32_t j = 0; j < nobs; ++j)
        if (cl[j] >= 0)
            members[cl[j]].push_back(j);
    uint32_t pos = 0;
    std::vector<double> xy;
    std::vector<int32_t> hull;
    for (uint32_t l = 0; l < K; ++l)
    {
        const auto& mem = members[l];
        xy.resize(2 * mem.size());
        float zmin = FLT_MAX, zmax = -FLT_MAX;
        for (size_t t = 0; t < mem.size(); ++t)
        {
            xy[2 * t] = obs[3 * mem[t]];
            xy[2 * t + 1] = obs[3 * mem[t] + 1];
            zmin = std::min(zmin, obs[3 * mem[t] + 2]);
            zmax = std::max(zmax, obs[3 * mem[t] + 2]);
        }
        hull.resize(mem.size() + 1);
        uint32_t hn = 0;
        lpo_convex_hull(xy.data(), static_cast<uint32_t>(mem.size()), hull.data(), &hn);
        out->hull_offsets[l] = pos;
        if (pos + hn > out->hull_capacity)
            return LP_ERR_CAPACITY;
        std::memcpy(out->hull_indices + pos, hull.data(), hn * sizeof(int32_t));
        pos += hn;
        if (out->z_min)
            out->z_min[l] = zmin;
        if (out->z_max)
            out->z_max[l] = zmax;
        if (cfg->compute_obb)
        {
            std::vector<double> hp(2 * static_cast<size_t>(hn));
            for (uint32_t t = 0; t < hn; ++t)
            {
                hp[2 * t] = xy[2 * hull[t]];
                hp[2 * t + 1] = xy[2 * hull[t] + 1];
            }
            if (out->obb_calipers)
                lpo_bounding_box_rotating_calipers(hp.data(), hn, &out->obb_calipers[l]);
            if (out->obb_pca)
                lpo_bounding_box_pca(hp.data(), hn, &out->obb_pca[l], nullptr);
        }
    }
    out->hull_offsets[K] = pos;
    out->n_hull_indices = pos;
    out->status = LP_OK;
    return LP_OK;
}

} // extern "C"

extern "C" {
// RANSAC index stream exactly as segmenter.cpp:369-386 draws it: std::mt19937{42} and
// std::uniform_int_distribution<uint32_t>{0, n - 1}; out receives 2 * iters indices (p2, p3).
void lpo_ransac_draws(uint32_t n, uint32_t iters, uint32_t* out)
{
    std::mt19937 gen{42};
    std::uniform_int_distribution<uint32_t> dist{0, n - 1U};
    for (uint32_t it = 0; it < iters; ++it)
    {
        const uint32_t a = dist(gen);
        uint32_t b = dist(gen);
        while (b == a && n > 1)
            b = dist(gen);
        out[2 * it] = a;
        out[2 * it + 1] = b;
    }
}
}

extern "C" {
// ---------------------------------------------------------------------------------------------
// The processor's per-cluster loop after the hulls: Processor::run, processor.cpp:609-797 (the
// clustered cloud with std::rand() colours, the vehicle gates, convertPolygonPointsToMarker).
// ---------------------------------------------------------------------------------------------

// glibc's rand() (random_r, TYPE_3 additive feedback generator), restated from its published
// algorithm: state r[0] = seed (1 when never seeded), r[i] = 16807 r[i-1] mod (2^31 - 1) for
// i = 1..30, r[31..33] = r[0..2], then r[i] = r[i-31] + r[i-3] mod 2^32; output k is r[k+344] >> 1
// (the first 310 values after r[33] are discarded by the seeding).
struct GlibcRand
{
    uint32_t w[34];
    uint64_t i = 34; // index of the next r[i]
    explicit GlibcRand(uint32_t seed = 1)
    {
        int32_t r[34];
        r[0] = static_cast<int32_t>(seed);
        for (int k = 1; k < 31; ++k)
        {
            const int64_t hi = r[k - 1] / 127773, lo = r[k - 1] % 127773;
            int64_t word = 16807 * lo - 2836 * hi;
            if (word < 0)
                word += 2147483647;
            r[k] = static_cast<int32_t>(word);
        }
        for (int k = 31; k < 34; ++k)
            r[k] = r[k - 31];
        for (int k = 0; k < 34; ++k)
            w[k] = static_cast<uint32_t>(r[k]);
        for (int k = 0; k < 310; ++k)
            step();
    }
    uint32_t step()
    {
        // ring of the last 34 values: r[i] = r[i-31] + r[i-3]
        const uint32_t v = w[(i - 31) % 34] + w[(i - 3) % 34];
        w[i % 34] = v;
        ++i;
        return v;
    }
    int32_t next() { return static_cast<int32_t>(step() >> 1); }
};

int32_t lpo_glibc_rand(uint64_t skip, uint32_t count, int32_t* out)
{
    GlibcRand g;
    for (uint64_t k = 0; k < skip; ++k)
        g.step();
    for (uint32_t k = 0; k < count; ++k)
        out[k] = g.next();
    return 0;
}

namespace
{
// processor.hpp:60-192: the vehicle table widened by the tolerances, its volume and area bounds and
// the overall limits, in the same binary64 expressions.
struct VehicleTable
{
    double dims[5][6]; // min/max length, width, height
    double bounds[5][4]; // min/max volume, area
    double min_h, max_h, min_v, max_v;
    VehicleTable()
    {
        const double base[5][6] = {{4.3, 4.6, 1.6, 1.9, 1.4, 1.5},
                                    {4.6, 5.0, 1.6, 1.9, 1.4, 1.5},
                                    {4.6, 5.2, 1.7, 2.1, 1.7, 1.8},
                                    {5.2, 5.8, 1.9, 2.2, 1.8, 2.0},
                                    {4.9, 5.2, 1.7, 2.1, 1.7, 1.8}};
        const double lt = 0.8, wt = 0.5, ht = 0.5;
        for (int v = 0; v < 5; ++v)
        {
            dims[v][0] = base[v][0] - lt;
            dims[v][1] = base[v][1] + lt;
            dims[v][2] = base[v][2] - wt;
            dims[v][3] = base[v][3] + wt;
            dims[v][4] = base[v][4] - ht;
            dims[v][5] = base[v][5] + ht;
        }
        for (int v = 0; v < 5; ++v)
        {
            bounds[v][0] = dims[v][0] * dims[v][2] * dims[v][4];
            bounds[v][1] = dims[v][1] * dims[v][3] * dims[v][5];
            bounds[v][2] = dims[v][0] * dims[v][2];
            bounds[v][3] = dims[v][1] * dims[v][3];
        }
        min_h = std::numeric_limits<double>::max();
        max_h = std::numeric_limits<double>::lowest();
        min_v = std::numeric_limits<double>::max();
        max_v = std::numeric_limits<double>::lowest();
        for (int v = 0; v < 5; ++v)
        {
            if (dims[v][4] < min_h)
                min_h = dims[v][4];
            if (dims[v][5] > max_h)
                max_h = dims[v][5];
            if (bounds[v][0] < min_v)
                min_v = bounds[v][0];
            if (bounds[v][1] > max_v)
                max_v = bounds[v][1];
        }
    }
};
} // namespace

lp_status lpo_cluster_objects(const float* xyzi, const int32_t* labels, uint32_t n, uint32_t K,
                              const uint32_t* hull_offsets, const int32_t* hull_indices, const float* zmin_in,
                              const float* zmax_in, const lp_object_config* cfg, lp_object_output* out)
{
    static const VehicleTable vt;
    GlibcRand g;
    for (uint64_t k = 0; k < cfg->rand_draws; ++k)
        g.step();
    uint32_t cpos = 0, mpos = 0;
    bool overflow = false;
    std::vector<std::vector<uint32_t>> members(K);
    for (uint32_t i = 0; i < n; ++i)
        if (labels[i] >= 0 && static_cast<uint32_t>(labels[i]) < K)
            members[labels[i]].push_back(i);
    std::vector<double> pts;
    for (uint32_t l = 0; l < K; ++l)
    {
        const uint8_t r = static_cast<uint8_t>(g.next() % 256), gg = static_cast<uint8_t>(g.next() % 256),
                      b = static_cast<uint8_t>(g.next() % 256);
        pts.clear();
        double z_min = std::numeric_limits<double>::max(), z_max = std::numeric_limits<double>::lowest();
        for (uint32_t i : members[l])
        {
            if (out->clustered_cloud)
                out->clustered_cloud[cpos] = lp_xyzrgb{xyzi[4 * i], xyzi[4 * i + 1], xyzi[4 * i + 2], r, gg, b, 255};
            ++cpos;
            pts.push_back(xyzi[4 * i]);
            pts.push_back(xyzi[4 * i + 1]);
            const double z = xyzi[4 * i + 2];
            if (z < z_min)
                z_min = z;
            if (z > z_max)
                z_max = z;
        }
        (void)zmin_in;
        (void)zmax_in;
        // polygon points in hull order
        std::vector<double> poly;
        for (uint32_t k = hull_offsets[l]; k < hull_offsets[l + 1]; ++k)
        {
            const uint32_t i = members[l][hull_indices[k]];
            poly.push_back(xyzi[4 * i]);
            poly.push_back(xyzi[4 * i + 1]);
        }
        int32_t cls = -1;
        lp_bounding_box gbox;
        std::memset(&gbox, 0, sizeof(gbox));
        const double height = z_max - z_min;
        const uint32_t np = static_cast<uint32_t>(poly.size() / 2);
        if (cfg->vehicle_gates && np >= 3 && members[l].size() > 150 && height > vt.min_h && height < vt.max_h)
        {
            // polygonArea (polygonizer.hpp:186-198)
            double area = 0.0;
            for (uint32_t k = 0; k + 1 < np; ++k)
                area += (poly[2 * k] * poly[2 * k + 3]) - (poly[2 * k + 2] * poly[2 * k + 1]);
            area += (poly[2 * (np - 1)] * poly[1]) - (poly[0] * poly[2 * (np - 1) + 1]);
            const double polygon_area = std::fabs(area) * 0.5;
            const double polygon_volume = polygon_area * height;
            if (polygon_volume > vt.min_v && polygon_volume < vt.max_v)
            {
                lpo_bounding_box_rotating_calipers(pts.data(), static_cast<uint32_t>(members[l].size()), &gbox);
                if (gbox.is_valid && polygon_area / gbox.area > 0.4)
                {
                    auto dist = [&](int a, int c) {
                        const double dx = gbox.corners[a][0] - gbox.corners[c][0];
                        const double dy = gbox.corners[a][1] - gbox.corners[c][1];
                        return std::sqrt(dx * dx + dy * dy);
                    };
                    const double e1 = dist(0, 1), e2 = dist(1, 2);
                    const double L = std::max(e1, e2), W = std::min(e1, e2);
                    for (int v = 0; v < 5; ++v)
                    {
                        const double* d = vt.dims[v];
                        const double* bb = vt.bounds[v];
                        if (L > d[0] && L < d[1] && W > d[2] && W < d[3] && height > d[4] && height < d[5] &&
                            polygon_volume > bb[0] && polygon_volume < bb[1] && polygon_area > bb[2] &&
                            polygon_area < bb[3])
                        {
                            cls = v;
                            poly.assign({gbox.corners[0][0], gbox.corners[0][1], gbox.corners[1][0], gbox.corners[1][1],
                                         gbox.corners[2][0], gbox.corners[2][1], gbox.corners[3][0], gbox.corners[3][1]});
                            break;
                        }
                    }
                }
            }
        }
        if (out->vehicle_class)
            out->vehicle_class[l] = cls;
        if (out->gate_boxes)
            out->gate_boxes[l] = gbox;
        if (out->marker_offsets)
            out->marker_offsets[l] = mpos;
        const uint32_t m = static_cast<uint32_t>(poly.size() / 2);
        if (m >= 3)
        {
            auto put = [&](double x, double y, double z) {
                if (out->marker_points && mpos < out->marker_capacity)
                {
                    out->marker_points[3 * static_cast<size_t>(mpos)] = x;
                    out->marker_points[3 * static_cast<size_t>(mpos) + 1] = y;
                    out->marker_points[3 * static_cast<size_t>(mpos) + 2] = z;
                }
                else if (out->marker_points)
                    overflow = true;
                ++mpos;
            };
            for (const double z : {z_min, z_max})
            {
                for (uint32_t k = 1; k < m; ++k)
                {
                    put(poly[2 * (k - 1)], poly[2 * (k - 1) + 1], z);
                    put(poly[2 * k], poly[2 * k + 1], z);
                }
                put(poly[2 * (m - 1)], poly[2 * (m - 1) + 1], z);
                put(poly[0], poly[1], z);
            }
            for (uint32_t k = 0; k < m; ++k)
            {
                put(poly[2 * k], poly[2 * k + 1], z_min);
                put(poly[2 * k], poly[2 * k + 1], z_max);
            }
        }
    }
    if (out->marker_offsets)
        out->marker_offsets[K] = mpos;
    out->n_clustered = cpos;
    out->n_marker_points = mpos;
    return overflow ? LP_ERR_CAPACITY : LP_OK;
}
}
