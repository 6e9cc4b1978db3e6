// lidar_processing_gpu.hpp — C++ drop-in classes over liblp_gpu.so's C ABI, with the reference
// library's class names, member signatures, label enums and exception types
// (lidar_processing_lib/include/lidar_processing_lib/{segmenter,noise_remover,clusterer,polygonizer}.hpp).
//
// Header-only; needs include/lidar_gb300.h and links against liblp_gpu.so. Point clouds are any
// type with a `.points` vector (pcl::PointCloud<P>), or a std::vector<P>, of structs exposing x, y,
// z (and `ring` for organised clouds), so pcl::PointCloud<pcl::PointXYZIR> works unchanged. Objects
// own a device context and, like the reference objects, are not thread-safe. The geometry helpers
// the processor node calls next to the classes (polygonArea, distance, ...; polygonizer.hpp:158-231)
// are here too, so a node can switch namespaces wholesale.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "lidar_gb300.h"

namespace lidar_processing_gpu
{
enum class Label : std::uint32_t
{
    UNKNOWN = 0,
    GROUND,
    OBSTACLE
};
enum class NoiseRemoverLabel : std::uint8_t
{
    VALID = 0,
    NOISE = 1
};
using ClusterLabel = std::int32_t;

enum class Orientation : std::uint8_t
{
    ANTICLOCKWISE = 0,
    CLOCKWISE = 1,
    COLINEAR = 2
};
enum class PolygonContour : std::uint8_t
{
    OPEN = 0,
    ENCLOSED = 1
};

struct PointXY
{
    double x;
    double y;
};
struct PointXYZ
{
    double x;
    double y;
    double z;
};
struct AntipodalPair
{
    std::int32_t index_1;
    std::int32_t index_2;
};
struct BoundingBox
{
    std::array<PointXY, 4> corners;
    float area;
    float angle_rad;
    bool is_valid;
};

// The jump-convolution colour image (Segmenter::image(), a CV_8UC3 cv::Mat in the reference).
struct Image
{
    int rows = 0;
    int cols = 0;
    std::vector<std::uint8_t> bgr; // rows * cols * 3
};

namespace detail
{
// Maps status codes onto the exceptions the reference throws for the same conditions.
inline void check(lp_status s, lp_context* ctx)
{
    if (s == LP_OK)
        return;
    std::string msg = lp_status_string(s);
    if (ctx)
    {
        const char* d = lp_last_error(ctx);
        if (d && *d)
            msg += std::string(": ") + d;
    }
    if (s == LP_ERR_CAPACITY)
        throw std::overflow_error(msg);
    if (s == LP_ERR_BAD_ARG)
        throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
}

class Context
{
  public:
    explicit Context(int device = 0)
    {
        check(lp_context_create(device, &ctx_), nullptr);
    }
    ~Context()
    {
        lp_context_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    lp_context* get() const noexcept
    {
        return ctx_;
    }

  private:
    lp_context* ctx_ = nullptr;
};

template <typename T, typename = void>
struct has_ring : std::false_type
{
};
template <typename T>
struct has_ring<T, std::void_t<decltype(std::declval<T>().ring)>> : std::true_type
{
};

template <typename Cloud>
auto& points_of(const Cloud& c)
{
    return c.points;
}
template <typename P, typename A>
const std::vector<P, A>& points_of(const std::vector<P, A>& v)
{
    return v;
}

template <typename Cloud>
void pack(const Cloud& cloud, std::vector<float>& xyzi, std::vector<std::uint16_t>* ring)
{
    const auto& pts = points_of(cloud);
    xyzi.resize(pts.size() * 4);
    using P = std::decay_t<decltype(pts[0])>;
    if constexpr (has_ring<P>::value)
        if (ring)
            ring->resize(pts.size());
    for (std::size_t i = 0; i < pts.size(); ++i)
    {
        xyzi[4 * i] = pts[i].x;
        xyzi[4 * i + 1] = pts[i].y;
        xyzi[4 * i + 2] = pts[i].z;
        xyzi[4 * i + 3] = 0.0f;
        if constexpr (has_ring<P>::value)
            if (ring)
                (*ring)[i] = pts[i].ring;
    }
}
} // namespace detail

// segmenter.hpp:87-112 (same field names and defaults)
struct SegmenterConfiguration
{
    float elevation_up_deg = 2.0F;
    float elevation_down_deg = -24.8F;
    std::int32_t image_width = 2048;
    std::int32_t image_height = 64;
    bool assume_unorganized_cloud = false;
    float grid_radial_spacing_m = 2.0F;
    float grid_slice_resolution_deg = 1.0F;
    float ground_height_threshold_m = 0.2F;
    float road_maximum_slope_m_per_m = 0.2F;
    float min_distance_m = 2.0F;
    float max_distance_m = 100.0F;
    float sensor_height_m = 1.73F;
    float kernel_threshold_distance_m = 1.0F;
    float amplification_factor = 5.0F;
    float z_min_m = -3.0F;
    float z_max_m = 4.0F;
    bool display_recm_with_low_confidence_points = false; // visualisation only; ignored
};

class Segmenter
{
  public:
    // segmenter.hpp:135-151 (the colour constants are the BGR triples of image())
    static constexpr float DEG_TO_RAD = static_cast<float>(M_PI / 180.0);
    static constexpr float TWO_M_PIf = static_cast<float>(2.0 * M_PI);
    static constexpr float INVALID_Z = std::numeric_limits<float>::max();
    static constexpr float INVALID_DEPTH_M = std::numeric_limits<float>::max();
    static constexpr std::int32_t INVALID_INDEX = -1;
    static constexpr std::array<std::uint8_t, 3> CV_OBSTACLE{0, 0, 255};
    static constexpr std::array<std::uint8_t, 3> CV_GROUND{0, 255, 0};
    static constexpr std::array<std::uint8_t, 3> CV_INTERSECTION_OR_UNKNOWN{0, 255, 255};
    static constexpr std::array<std::uint8_t, 3> CV_INTERSECTION{255, 0, 0};
    static constexpr std::array<std::uint8_t, 3> CV_UNKNOWN{255, 255, 255};
    static constexpr std::uint32_t MAX_CLOUD_SIZE = 200'000U;

    explicit Segmenter(int device = 0) : ctx_(device) {}

    void config(const SegmenterConfiguration& config)
    {
        config_ = config;
    }
    const SegmenterConfiguration& config() const noexcept
    {
        return config_;
    }
    const Image& image() const noexcept
    {
        return image_;
    }

    // Segmenter::segment (segmenter.cpp:87-101): labels are assigned, one per input point.
    template <typename Cloud>
    void segment(const Cloud& cloud, std::vector<Label>& labels)
    {
        detail::pack(cloud, xyzi_, &ring_);
        using P = std::decay_t<decltype(detail::points_of(cloud)[0])>;
        const std::uint16_t* ring = detail::has_ring<P>::value ? ring_.data() : nullptr;
        const std::uint32_t n = static_cast<std::uint32_t>(xyzi_.size() / 4);
        const lp_segmenter_config c = raw();
        labels.assign(n, Label::UNKNOWN);
        image_.rows = c.image_height;
        image_.cols = c.image_width;
        image_.bgr.assign(static_cast<std::size_t>(c.image_height) * c.image_width * 3, 0);
        detail::check(lp_segment(ctx_.get(), xyzi_.data(), ring, n, &c, reinterpret_cast<std::uint32_t*>(labels.data()),
                                 image_.bgr.data()),
                      ctx_.get());
    }

  private:
    lp_segmenter_config raw() const
    {
        lp_segmenter_config c;
        c.elevation_up_deg = config_.elevation_up_deg;
        c.elevation_down_deg = config_.elevation_down_deg;
        c.image_width = config_.image_width;
        c.image_height = config_.image_height;
        c.assume_unorganized_cloud = config_.assume_unorganized_cloud ? 1 : 0;
        c.grid_radial_spacing_m = config_.grid_radial_spacing_m;
        c.grid_slice_resolution_deg = config_.grid_slice_resolution_deg;
        c.ground_height_threshold_m = config_.ground_height_threshold_m;
        c.road_maximum_slope_m_per_m = config_.road_maximum_slope_m_per_m;
        c.min_distance_m = config_.min_distance_m;
        c.max_distance_m = config_.max_distance_m;
        c.sensor_height_m = config_.sensor_height_m;
        c.kernel_threshold_distance_m = config_.kernel_threshold_distance_m;
        c.amplification_factor = config_.amplification_factor;
        c.z_min_m = config_.z_min_m;
        c.z_max_m = config_.z_max_m;
        return c;
    }

    detail::Context ctx_;
    SegmenterConfiguration config_;
    Image image_;
    std::vector<float> xyzi_;
    std::vector<std::uint16_t> ring_;
};

// noise_remover.hpp:41-54
struct NoiseRemoverConfiguration
{
    float radius_multiplier_m_per_m = 0.02F;
    float min_search_radius_m = 0.1F;
    std::uint32_t min_neighbours = 4U;
};

class NoiseRemover
{
  public:
    using PointT = std::array<float, 3>;
    explicit NoiseRemover(int device = 0) : ctx_(device) {}
    void reserve(std::uint32_t) {}
    void config(const NoiseRemoverConfiguration& config)
    {
        config_ = config;
    }
    const NoiseRemoverConfiguration& config() const noexcept
    {
        return config_;
    }

    // NoiseRemover::filter (noise_remover.cpp:38-68)
    void filter(const std::vector<PointT>& points, std::vector<NoiseRemoverLabel>& labels)
    {
        labels.assign(points.size(), NoiseRemoverLabel::VALID);
        const lp_noise_remover_config c{config_.radius_multiplier_m_per_m, config_.min_search_radius_m,
                                        config_.min_neighbours};
        detail::check(lp_noise_remove(ctx_.get(), points.empty() ? nullptr : points[0].data(), 3,
                                      static_cast<std::uint32_t>(points.size()), &c,
                                      reinterpret_cast<std::uint8_t*>(labels.data())),
                      ctx_.get());
    }

  private:
    detail::Context ctx_;
    NoiseRemoverConfiguration config_;
};

// clusterer.hpp:61-68
struct ClustererConfiguration
{
    float voxel_grid_range_resolution_m = 0.4F;
    float voxel_grid_azimuth_resolution_deg = 1.0F;
    float voxel_grid_elevation_resolution_deg = 1.5F;
    std::uint32_t min_cluster_size = 3;
};

class Clusterer
{
  public:
    static constexpr float TWO_M_PIf = static_cast<float>(2.0 * M_PI);
    static constexpr float DEG_TO_RAD = static_cast<float>(M_PI / 180.0);
    static constexpr std::int32_t INVALID_LABEL = -1;
    explicit Clusterer(int device = 0) : ctx_(device) {}
    void config(const ClustererConfiguration& config)
    {
        config_ = config;
    }
    const ClustererConfiguration& config() const noexcept
    {
        return config_;
    }

    // Clusterer::cluster (clusterer.cpp:43-53); throws std::overflow_error past 200,000 voxels
    template <typename Cloud>
    void cluster(const Cloud& cloud, std::vector<ClusterLabel>& labels)
    {
        detail::pack(cloud, xyzi_, nullptr);
        const std::uint32_t n = static_cast<std::uint32_t>(xyzi_.size() / 4);
        labels.assign(n, INVALID_LABEL);
        const lp_clusterer_config c{config_.voxel_grid_range_resolution_m, config_.voxel_grid_azimuth_resolution_deg,
                                    config_.voxel_grid_elevation_resolution_deg, config_.min_cluster_size};
        detail::check(lp_cluster(ctx_.get(), xyzi_.data(), 4, n, &c, labels.data()), ctx_.get());
    }

  private:
    detail::Context ctx_;
    ClustererConfiguration config_;
    std::vector<float> xyzi_;
};

// polygonizer.hpp:54-60; the reference sizes its scratch from max_points and reads nothing else
struct PolygonizerConfiguration
{
    Orientation orientation = Orientation::ANTICLOCKWISE;
    PolygonContour contour = PolygonContour::OPEN;
    std::uint32_t max_points = 100'000;
};

class Polygonizer
{
  public:
    explicit Polygonizer(int device = 0) : ctx_(device) {}

    void config(const PolygonizerConfiguration& config)
    {
        config_ = config;
    }
    const PolygonizerConfiguration& config() const noexcept
    {
        return config_;
    }

    // Polygonizer::concaveHull (polygonizer.hpp:233-237) has an empty body: indices are left as given.
    template <typename PointT>
    void concaveHull(const std::vector<PointT>&, std::vector<std::int32_t>&)
    {
    }

    // Polygonizer::convexHull (polygonizer.cpp:33-91): counter-clockwise hull indices
    template <typename PointT>
    void convexHull(const std::vector<PointT>& points, std::vector<std::int32_t>& indices)
    {
        xy_.resize(points.size() * 2);
        for (std::size_t i = 0; i < points.size(); ++i)
        {
            xy_[2 * i] = points[i].x;
            xy_[2 * i + 1] = points[i].y;
        }
        indices.resize(points.size() + 1);
        std::uint32_t h = 0;
        detail::check(lp_convex_hull(ctx_.get(), xy_.data(), static_cast<std::uint32_t>(points.size()), indices.data(), &h),
                      ctx_.get());
        indices.resize(h);
    }

    void findAntipodalPairsOfConvexHull(const std::vector<PointXY>& hull, std::vector<AntipodalPair>& pairs)
    {
        pairs.resize(4 * hull.size() + 16);
        std::uint32_t np = 0;
        detail::check(lp_antipodal_pairs(ctx_.get(), reinterpret_cast<const double*>(hull.data()),
                                         static_cast<std::uint32_t>(hull.size()),
                                         reinterpret_cast<std::int32_t*>(pairs.data()),
                                         static_cast<std::uint32_t>(pairs.size()), &np),
                      ctx_.get());
        pairs.resize(np);
    }

    BoundingBox boundingBoxRotatingCalipers(const std::vector<PointXY>& hull)
    {
        lp_bounding_box b;
        detail::check(lp_bounding_box_rotating_calipers(ctx_.get(), reinterpret_cast<const double*>(hull.data()),
                                                        static_cast<std::uint32_t>(hull.size()), &b),
                      ctx_.get());
        return convert(b);
    }

    BoundingBox boundingBoxPrincipalComponentAnalysis(const std::vector<PointXY>& hull)
    {
        lp_bounding_box b;
        detail::check(lp_bounding_box_pca(ctx_.get(), reinterpret_cast<const double*>(hull.data()),
                                          static_cast<std::uint32_t>(hull.size()), &b),
                      ctx_.get());
        return convert(b);
    }

  private:
    static BoundingBox convert(const lp_bounding_box& b)
    {
        BoundingBox r{};
        for (int k = 0; k < 4; ++k)
            r.corners[k] = {b.corners[k][0], b.corners[k][1]};
        r.area = b.area;
        r.angle_rad = b.angle_rad;
        r.is_valid = b.is_valid != 0;
        return r;
    }

    detail::Context ctx_;
    PolygonizerConfiguration config_;
    std::vector<double> xy_;
};

// Geometry helpers of polygonizer.hpp:158-231, in the same arithmetic (double, same operation order).
template <typename PointT>
inline Orientation orientation(const PointT& a, const PointT& b, const PointT& c) noexcept
{
    const auto turn = (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
    return turn > 0.0 ? Orientation::ANTICLOCKWISE : (turn < 0.0 ? Orientation::CLOCKWISE : Orientation::COLINEAR);
}

template <typename PointT>
inline auto crossProduct(const PointT& a, const PointT& b) noexcept
{
    return (a.x * b.y) - (b.x * a.y);
}

// Shoelace area of a polygon given as its vertices in order (0 below three vertices).
template <typename PointT>
inline double polygonArea(const std::vector<PointT>& v) noexcept
{
    const std::size_t n = v.size();
    if (n < 3)
        return 0.0;
    double twice = 0.0;
    for (std::size_t i = 0; i + 1 < n; ++i)
        twice += crossProduct(v[i], v[i + 1]);
    twice += crossProduct(v[n - 1], v[0]);
    return std::fabs(twice) * 0.5;
}

template <typename PointT>
inline double distanceSquared(const PointT& a, const PointT& b) noexcept
{
    const double dx = a.x - b.x;
    const double dy = a.y - b.y;
    return dx * dx + dy * dy;
}

template <typename PointT>
inline double distance(const PointT& a, const PointT& b) noexcept
{
    return std::sqrt(distanceSquared(a, b));
}

// Area of a rectangle from three consecutive corners (the fourth is not read).
template <typename PointT>
inline double areaOfRectangle(const PointT& a, const PointT& b, const PointT& c, const PointT&) noexcept
{
    return std::sqrt(distanceSquared(a, b) * distanceSquared(b, c));
}

template <typename PointT>
inline double areaOfTriangle(const PointT& a, const PointT& b, const PointT& c) noexcept
{
    return std::fabs((a.x * (b.y - c.y) + b.x * (c.y - a.y) + c.x * (a.y - b.y)) * 0.5);
}

static_assert(sizeof(PointXY) == 16, "PointXY must be two packed doubles (lp_* take n x 2 doubles)");
static_assert(sizeof(AntipodalPair) == 8, "AntipodalPair must be two int32 (lp_antipodal_pairs layout)");
} // namespace lidar_processing_gpu
