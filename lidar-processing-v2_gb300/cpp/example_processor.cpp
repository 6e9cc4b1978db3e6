// example_processor.cpp — Processor::run's perception sequence (src/processor/src/processor.cpp:
// 552-671) written against the drop-in classes of lidar_processing_gpu.hpp: segment the cloud,
// take the OBSTACLE points in input order, cluster them, gather each cluster in input order and
// hull it. Prints one line of counts and a checksum of all labels and hull indices.
//
//   example_processor <xyzi.bin> [rings.bin] [image_height image_width]
// xyzi.bin holds n x 4 float32 (x, y, z, intensity); rings.bin n uint16 ring indices.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "lidar_processing_gpu.hpp"

// Stand-ins for pcl::PointXYZIR, pcl::PointXYZ and pcl::PointCloud (same fields). They live in
// their own namespace, as PCL's do: the drop-in namespace has a PointXYZ of its own (doubles, the
// polygonizer's point type), exactly like lidar_processing_lib.
namespace sensor
{
struct PointXYZIR
{
    float x, y, z, intensity;
    std::uint16_t ring;
};
struct PointXYZ
{
    float x, y, z;
};
template <typename P>
struct Cloud
{
    std::vector<P> points;
};
} // namespace sensor

namespace
{

template <typename T>
std::vector<T> read_all(const char* path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<T> v(static_cast<std::size_t>(f.tellg()) / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
    return v;
}
} // namespace

int main(int argc, char** argv)
{
    using namespace lidar_processing_gpu;
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: %s xyzi.bin [rings.bin] [image_height image_width]\n", argv[0]);
        return 2;
    }
    const std::vector<float> raw = read_all<float>(argv[1]);
    const std::vector<std::uint16_t> rings = (argc > 2) ? read_all<std::uint16_t>(argv[2]) : std::vector<std::uint16_t>{};
    sensor::Cloud<sensor::PointXYZIR> cloud;
    cloud.points.resize(raw.size() / 4);
    for (std::size_t i = 0; i < cloud.points.size(); ++i)
        cloud.points[i] = {raw[4 * i], raw[4 * i + 1], raw[4 * i + 2], raw[4 * i + 3],
                           rings.empty() ? std::uint16_t{0} : rings[i]};

    SegmenterConfiguration sc;
    if (argc > 4)
    {
        sc.image_height = std::atoi(argv[3]);
        sc.image_width = std::atoi(argv[4]);
    }
    Segmenter segmenter;
    segmenter.config(sc);
    std::vector<Label> labels;
    segmenter.segment(cloud, labels);

    sensor::Cloud<sensor::PointXYZ> obstacles;
    std::size_t ground = 0;
    for (std::size_t i = 0; i < labels.size(); ++i)
    {
        if (labels[i] == Label::GROUND)
            ++ground;
        else if (labels[i] == Label::OBSTACLE)
            obstacles.points.push_back({cloud.points[i].x, cloud.points[i].y, cloud.points[i].z});
    }

    ClustererConfiguration cc;
    cc.voxel_grid_elevation_resolution_deg = 3.0F; // processor.param.yaml:34
    Clusterer clusterer;
    clusterer.config(cc);
    std::vector<ClusterLabel> cl;
    clusterer.cluster(obstacles, cl);

    std::int32_t max_label = -1;
    for (const auto l : cl)
        max_label = std::max(max_label, l);
    Polygonizer polygonizer;
    std::vector<PointXY> pts;
    std::vector<std::int32_t> hull;
    std::uint64_t checksum = 1469598103934665603ull;
    auto mix = [&checksum](std::uint64_t v) { checksum = (checksum ^ v) * 1099511628211ull; };
    for (const auto l : labels)
        mix(static_cast<std::uint32_t>(l));
    for (const auto l : cl)
        mix(static_cast<std::uint32_t>(l));
    std::size_t hull_total = 0;
    for (std::int32_t label = 0; label <= max_label; ++label)
    {
        pts.clear();
        for (std::size_t j = 0; j < cl.size(); ++j)
            if (cl[j] == label)
                pts.push_back({obstacles.points[j].x, obstacles.points[j].y});
        polygonizer.convexHull(pts, hull);
        hull_total += hull.size();
        for (const auto h : hull)
            mix(static_cast<std::uint32_t>(h));
    }
    std::printf("points %zu ground %zu obstacles %zu clusters %d hull_vertices %zu checksum %016llx\n",
                cloud.points.size(), ground, obstacles.points.size(), max_label + 1, hull_total,
                static_cast<unsigned long long>(checksum));
    return 0;
}
