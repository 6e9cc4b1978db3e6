// C entry points over the REFERENCE library's own classes (Segmenter, NoiseRemover, Clusterer,
// Polygonizer), compiled from the reference sources against the stand-in headers in
// oracle/shim/. Test infrastructure only: it is the arbiter that pins the oracle restatement
// (oracle/lp_oracle.c) and generates the golden fixtures under tests/golden/. Built by
// oracle/build_ref.sh into oracle/_ref/ where the reference tree is available; never shipped.
//
// Function names mirror include/lidar_gb300.h with the prefix `lpr_`.
#include "lidar_gb300.h"

#include "lidar_processing_lib/clusterer.hpp"
#include "lidar_processing_lib/noise_remover.hpp"
#include "lidar_processing_lib/polygonizer.hpp"
#include "lidar_processing_lib/segmenter.hpp"

#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <vector>

using namespace lidar_processing_lib;

namespace
{
struct QuietCerr
{
    std::stringstream sink;
    std::streambuf* old;
    QuietCerr() : old(std::cerr.rdbuf(sink.rdbuf())) {}
    ~QuietCerr() { std::cerr.rdbuf(old); }
};

SegmenterConfiguration toRef(const lp_segmenter_config& c)
{
    SegmenterConfiguration r;
    r.elevation_up_deg = c.elevation_up_deg;
    r.elevation_down_deg = c.elevation_down_deg;
    r.image_width = c.image_width;
    r.image_height = c.image_height;
    r.assume_unorganized_cloud = c.assume_unorganized_cloud != 0;
    r.grid_radial_spacing_m = c.grid_radial_spacing_m;
    r.grid_slice_resolution_deg = c.grid_slice_resolution_deg;
    r.ground_height_threshold_m = c.ground_height_threshold_m;
    r.road_maximum_slope_m_per_m = c.road_maximum_slope_m_per_m;
    r.min_distance_m = c.min_distance_m;
    r.max_distance_m = c.max_distance_m;
    r.sensor_height_m = c.sensor_height_m;
    r.kernel_threshold_distance_m = c.kernel_threshold_distance_m;
    r.amplification_factor = c.amplification_factor;
    r.z_min_m = c.z_min_m;
    r.z_max_m = c.z_max_m;
    r.display_recm_with_low_confidence_points = false;
    return r;
}

Segmenter& segmenter()
{
    static thread_local Segmenter* s = nullptr;
    if (!s)
    {
        QuietCerr q;
        s = new Segmenter();
    }
    return *s;
}

template <typename PointT>
void runSegment(const float* xyzi, const uint16_t* ring, uint32_t n, const lp_segmenter_config& cfg,
                uint32_t* labels_out, uint8_t* image_out)
{
    pcl::PointCloud<PointT> cloud;
    cloud.points.resize(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        cloud.points[i].x = xyzi[4 * i + 0];
        cloud.points[i].y = xyzi[4 * i + 1];
        cloud.points[i].z = xyzi[4 * i + 2];
        if constexpr (HasRing<PointT>::value)
        {
            cloud.points[i].ring = ring[i];
        }
    }
    Segmenter& s = segmenter();
    {
        QuietCerr q;
        s.config(toRef(cfg));
    }
    std::vector<Label> labels;
    s.segment(cloud, labels);
    for (uint32_t i = 0; i < n; ++i)
    {
        labels_out[i] = static_cast<uint32_t>(labels[i]);
    }
    if (image_out)
    {
        const cv::Mat& img = s.image();
        std::memcpy(image_out, img.buf.data(), img.buf.size());
    }
}

std::vector<PointXY> toXY(const double* xy, uint32_t n)
{
    std::vector<PointXY> pts(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        pts[i] = {xy[2 * i], xy[2 * i + 1]};
    }
    return pts;
}

void copyBox(const BoundingBox& b, lp_bounding_box* out)
{
    std::memset(out, 0, sizeof(*out));
    out->is_valid = b.is_valid ? 1 : 0;
    if (!b.is_valid)
    {
        return;
    }
    for (int k = 0; k < 4; ++k)
    {
        out->corners[k][0] = b.corners[k].x;
        out->corners[k][1] = b.corners[k].y;
    }
    out->area = b.area;
    out->angle_rad = b.angle_rad;
}
} // namespace

extern "C" {

lp_status lpr_segment(const float* xyzi, const uint16_t* ring, uint32_t n,
                      const lp_segmenter_config* cfg, uint32_t* labels_out, uint8_t* image_out)
{
    try
    {
        if (ring)
            runSegment<pcl::PointXYZIR>(xyzi, ring, n, *cfg, labels_out, image_out);
        else
            runSegment<pcl::PointXYZI>(xyzi, nullptr, n, *cfg, labels_out, image_out);
    }
    catch (const std::exception&)
    {
        return LP_ERR_INTERNAL;
    }
    return LP_OK;
}

lp_status lpr_noise_remove(const float* xyz, uint32_t stride, uint32_t n,
                           const lp_noise_remover_config* cfg, uint8_t* labels_out)
{
    try
    {
        // A fresh object per call: the reference kd-tree keeps its radius-search stack between
        // queries, so results depend on the object's history; one object per scan keeps the
        // per-scan result reproducible.
        NoiseRemover nr;
        NoiseRemoverConfiguration c;
        c.radius_multiplier_m_per_m = cfg->radius_multiplier_m_per_m;
        c.min_search_radius_m = cfg->min_search_radius_m;
        c.min_neighbours = cfg->min_neighbours;
        nr.config(c);
        nr.reserve(n);
        std::vector<NoiseRemover::PointT> pts(n);
        for (uint32_t i = 0; i < n; ++i)
        {
            pts[i] = {xyz[stride * i], xyz[stride * i + 1], xyz[stride * i + 2]};
        }
        std::vector<NoiseRemoverLabel> labels;
        nr.filter(pts, labels);
        for (uint32_t i = 0; i < n; ++i)
        {
            labels_out[i] = static_cast<uint8_t>(labels[i]);
        }
    }
    catch (const std::exception&)
    {
        return LP_ERR_INTERNAL;
    }
    return LP_OK;
}

lp_status lpr_cluster(const float* xyz, uint32_t stride, uint32_t n, const lp_clusterer_config* cfg,
                      int32_t* labels_out)
{
    try
    {
        static thread_local Clusterer* cl = nullptr;
        if (!cl)
            cl = new Clusterer();
        ClustererConfiguration c;
        c.voxel_grid_range_resolution_m = cfg->voxel_grid_range_resolution_m;
        c.voxel_grid_azimuth_resolution_deg = cfg->voxel_grid_azimuth_resolution_deg;
        c.voxel_grid_elevation_resolution_deg = cfg->voxel_grid_elevation_resolution_deg;
        c.min_cluster_size = cfg->min_cluster_size;
        cl->config(c);
        pcl::PointCloud<pcl::PointXYZRGB> cloud;
        cloud.points.reserve(n);
        for (uint32_t i = 0; i < n; ++i)
        {
            cloud.emplace_back(xyz[stride * i], xyz[stride * i + 1], xyz[stride * i + 2], 200, 0, 0);
        }
        std::vector<ClusterLabel> labels;
        cl->cluster(cloud, labels);
        for (uint32_t i = 0; i < n; ++i)
        {
            labels_out[i] = labels[i];
        }
    }
    catch (const std::overflow_error&)
    {
        return LP_ERR_CAPACITY;
    }
    catch (const std::exception&)
    {
        return LP_ERR_INTERNAL;
    }
    return LP_OK;
}

static Polygonizer& polygonizer()
{
    static thread_local Polygonizer* p = nullptr;
    if (!p)
        p = new Polygonizer();
    return *p;
}

lp_status lpr_convex_hull(const double* xy, uint32_t n, int32_t* indices_out, uint32_t* n_out)
{
    std::vector<PointXY> pts = toXY(xy, n);
    std::vector<int32_t> idx;
    polygonizer().convexHull(pts, idx);
    for (size_t i = 0; i < idx.size(); ++i)
        indices_out[i] = idx[i];
    *n_out = static_cast<uint32_t>(idx.size());
    return LP_OK;
}

lp_status lpr_antipodal_pairs(const double* xy, uint32_t n, int32_t* pairs_out, uint32_t capacity,
                              uint32_t* n_pairs)
{
    std::vector<PointXY> pts = toXY(xy, n);
    std::vector<AntipodalPair> pairs;
    polygonizer().findAntipodalPairsOfConvexHull(pts, pairs);
    *n_pairs = static_cast<uint32_t>(pairs.size());
    if (pairs.size() > capacity)
        return LP_ERR_CAPACITY;
    for (size_t i = 0; i < pairs.size(); ++i)
    {
        pairs_out[2 * i] = pairs[i].index_1;
        pairs_out[2 * i + 1] = pairs[i].index_2;
    }
    return LP_OK;
}

lp_status lpr_bounding_box_rotating_calipers(const double* xy, uint32_t n, lp_bounding_box* out)
{
    copyBox(polygonizer().boundingBoxRotatingCalipers(toXY(xy, n)), out);
    return LP_OK;
}

lp_status lpr_bounding_box_pca(const double* xy, uint32_t n, lp_bounding_box* out)
{
    copyBox(polygonizer().boundingBoxPrincipalComponentAnalysis(toXY(xy, n)), out);
    return LP_OK;
}

// Processor::run restated over the reference classes (processor.cpp:552-671), with the
// optional DROR pass on the input cloud that the processor declares (processor.hpp:243-246).
lp_status lpr_process_scan(const lp_pipeline_config* cfg, const lp_scan_input* scan,
                           lp_scan_output* out)
{
    const uint32_t n = scan->n;
    std::vector<uint8_t> noise(n, LP_NOISE_VALID);
    if (cfg->enable_noise_removal)
    {
        lp_status st = lpr_noise_remove(scan->xyzi, 4, n, &cfg->noise, noise.data());
        if (st != LP_OK)
            return st;
    }
    if (cfg->compute_ring)
        return LP_ERR_BAD_ARG; // the ring partition lives in the ROS dataloader node
    std::vector<uint32_t> keep;
    keep.reserve(n);
    for (uint32_t i = 0; i < n; ++i)
        if (noise[i] == LP_NOISE_VALID)
            keep.push_back(i);
    std::vector<float> xyzi(keep.size() * 4);
    std::vector<uint16_t> ring(scan->ring ? keep.size() : 0);
    for (size_t j = 0; j < keep.size(); ++j)
    {
        std::memcpy(&xyzi[4 * j], &scan->xyzi[4 * keep[j]], 16);
        if (scan->ring)
            ring[j] = scan->ring[keep[j]];
    }
    std::vector<uint32_t> seg(keep.size());
    lp_status st = lpr_segment(xyzi.data(), scan->ring ? ring.data() : nullptr,
                               static_cast<uint32_t>(keep.size()), &scan->seg, seg.data(), nullptr);
    if (st != LP_OK)
        return st;
    std::vector<uint32_t> obstacle; // input-point index of each obstacle point
    std::vector<float> obs_xyz;
    for (size_t j = 0; j < keep.size(); ++j)
    {
        if (seg[j] == LP_LABEL_OBSTACLE)
        {
            obstacle.push_back(keep[j]);
            obs_xyz.push_back(xyzi[4 * j]);
            obs_xyz.push_back(xyzi[4 * j + 1]);
            obs_xyz.push_back(xyzi[4 * j + 2]);
        }
    }
    const uint32_t nobs = static_cast<uint32_t>(obstacle.size());
    std::vector<int32_t> cl(nobs);
    if (nobs > 0)
    {
        st = lpr_cluster(obs_xyz.data(), 3, nobs, &cfg->cluster, cl.data());
        if (st != LP_OK)
            return st;
    }
    if (out->noise_labels)
        std::memcpy(out->noise_labels, noise.data(), n);
    if (out->seg_labels)
    {
        for (uint32_t i = 0; i < n; ++i)
            out->seg_labels[i] = LP_LABEL_UNKNOWN;
        for (size_t j = 0; j < keep.size(); ++j)
            out->seg_labels[keep[j]] = seg[j];
    }
    if (out->cluster_labels)
    {
        for (uint32_t i = 0; i < n; ++i)
            out->cluster_labels[i] = LP_INVALID_CLUSTER;
        for (uint32_t j = 0; j < nobs; ++j)
            out->cluster_labels[obstacle[j]] = cl[j];
    }
    int32_t max_label = -1;
    for (uint32_t j = 0; j < nobs; ++j)
        max_label = std::max(max_label, cl[j]);
    const uint32_t k = static_cast<uint32_t>(max_label + 1);
    out->n_obstacles = nobs;
    out->n_clusters = k;
    if (k > out->cluster_capacity)
        return LP_ERR_CAPACITY;
    uint32_t hull_pos = 0;
    std::vector<PointXY> pts;
    std::vector<int32_t> hull;
    for (uint32_t label = 0; label < k; ++label)
    {
        pts.clear();
        double zmin = std::numeric_limits<double>::max();
        double zmax = std::numeric_limits<double>::lowest();
        for (uint32_t j = 0; j < nobs; ++j)
        {
            if (cl[j] == static_cast<int32_t>(label))
            {
                pts.push_back({obs_xyz[3 * j], obs_xyz[3 * j + 1]});
                const double z = obs_xyz[3 * j + 2];
                if (z < zmin)
                    zmin = z;
                if (z > zmax)
                    zmax = z;
            }
        }
        polygonizer().convexHull(pts, hull);
        out->hull_offsets[label] = hull_pos;
        if (hull_pos + hull.size() > out->hull_capacity)
            return LP_ERR_CAPACITY;
        for (size_t h = 0; h < hull.size(); ++h)
            out->hull_indices[hull_pos + h] = hull[h];
        hull_pos += static_cast<uint32_t>(hull.size());
        if (out->z_min)
            out->z_min[label] = static_cast<float>(zmin);
        if (out->z_max)
            out->z_max[label] = static_cast<float>(zmax);
        if (cfg->compute_obb)
        {
            std::vector<PointXY> hp;
            for (int32_t h : hull)
                hp.push_back(pts[h]);
            if (out->obb_calipers)
                copyBox(polygonizer().boundingBoxRotatingCalipers(hp), &out->obb_calipers[label]);
            if (out->obb_pca)
                copyBox(polygonizer().boundingBoxPrincipalComponentAnalysis(hp), &out->obb_pca[label]);
        }
    }
    out->hull_offsets[k] = hull_pos;
    out->n_hull_indices = hull_pos;
    out->status = LP_OK;
    return LP_OK;
}

} // extern "C"
