"""The C++ drop-in header (lidar-processing-v2_gb300/cpp/lidar_processing_gpu.hpp) on CPU: it
compiles for every point type the reference library instantiates its templates with
(segmenter.hpp:264-271, clusterer.hpp:181-188, polygonizer.hpp:240-243), links against
liblp_gpu.so, maps a missing device onto std::runtime_error, and its geometry helpers give the
reference's values."""
import os
import subprocess

import lp_testlib as T

PKG = os.path.join(T.REPO, "lidar-processing-v2_gb300")

PROGRAM = r"""
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "lidar_processing_gpu.hpp"

// Stand-ins with the field layout of PCL's point types and of point_types.hpp's XYZR / XYZIR.
namespace pcl
{
struct PointXYZ { float x, y, z; };
struct PointXYZI { float x, y, z, intensity; };
struct PointXYZR { float x, y, z; std::uint16_t ring; };
struct PointXYZIR { float x, y, z, intensity; std::uint16_t ring; };
struct PointXYZRGB { float x, y, z; std::uint8_t r, g, b; };
template <class P> struct PointCloud { std::vector<P> points; };
}

namespace lp = lidar_processing_gpu;

template void lp::Segmenter::segment(const pcl::PointCloud<pcl::PointXYZ>&, std::vector<lp::Label>&);
template void lp::Segmenter::segment(const pcl::PointCloud<pcl::PointXYZI>&, std::vector<lp::Label>&);
template void lp::Segmenter::segment(const pcl::PointCloud<pcl::PointXYZR>&, std::vector<lp::Label>&);
template void lp::Segmenter::segment(const pcl::PointCloud<pcl::PointXYZIR>&, std::vector<lp::Label>&);
template void lp::Clusterer::cluster(const pcl::PointCloud<pcl::PointXYZ>&, std::vector<lp::ClusterLabel>&);
template void lp::Clusterer::cluster(const pcl::PointCloud<pcl::PointXYZI>&, std::vector<lp::ClusterLabel>&);
template void lp::Clusterer::cluster(const pcl::PointCloud<pcl::PointXYZRGB>&, std::vector<lp::ClusterLabel>&);
template void lp::Clusterer::cluster(const std::vector<pcl::PointXYZI>&, std::vector<lp::ClusterLabel>&);
template void lp::Polygonizer::convexHull(const std::vector<lp::PointXY>&, std::vector<std::int32_t>&);
template void lp::Polygonizer::convexHull(const std::vector<lp::PointXYZ>&, std::vector<std::int32_t>&);

static_assert(lp::detail::has_ring<pcl::PointXYZR>::value && lp::detail::has_ring<pcl::PointXYZIR>::value, "ring");
static_assert(!lp::detail::has_ring<pcl::PointXYZI>::value, "no ring");
static_assert(sizeof(lp::Label) == 4 && sizeof(lp::NoiseRemoverLabel) == 1, "label widths of the C ABI");
static_assert(std::is_same<lp::NoiseRemover::PointT, std::array<float, 3>>::value, "KDTree<float, 3>::PointT");

int main()
{
    int bad = 0;
    auto expect = [&](bool ok, const char* what) {
        if (!ok)
        {
            std::printf("FAIL %s\n", what);
            ++bad;
        }
    };
    const std::vector<lp::PointXY> square{{0, 0}, {2, 0}, {2, 2}, {0, 2}};
    expect(lp::polygonArea(square) == 4.0, "polygonArea square");
    expect(lp::polygonArea(std::vector<lp::PointXY>{{0, 0}, {1, 1}}) == 0.0, "polygonArea below three vertices");
    expect(lp::polygonArea(std::vector<lp::PointXY>{{0, 0}, {0, 2}, {2, 2}, {2, 0}}) == 4.0, "polygonArea clockwise");
    expect(lp::distance(lp::PointXY{0, 0}, lp::PointXY{3, 4}) == 5.0, "distance");
    expect(lp::distanceSquared(lp::PointXY{1, 1}, lp::PointXY{4, 5}) == 25.0, "distanceSquared");
    expect(lp::areaOfRectangle(square[0], square[1], square[2], square[3]) == 4.0, "areaOfRectangle");
    expect(lp::areaOfTriangle(square[0], square[1], square[2]) == 2.0, "areaOfTriangle");
    expect(lp::crossProduct(lp::PointXY{1, 0}, lp::PointXY{0, 1}) == 1.0, "crossProduct");
    expect(lp::orientation(square[0], square[1], square[2]) == lp::Orientation::ANTICLOCKWISE, "ccw");
    expect(lp::orientation(square[0], square[2], square[1]) == lp::Orientation::CLOCKWISE, "cw");
    expect(lp::orientation(square[0], lp::PointXY{1, 1}, square[2]) == lp::Orientation::COLINEAR, "colinear");
    expect(lp::Segmenter::MAX_CLOUD_SIZE == 200000u && lp::Clusterer::INVALID_LABEL == -1, "constants");
    try
    {
        lp::Segmenter seg;
        pcl::PointCloud<pcl::PointXYZIR> cloud;
        std::vector<lp::Label> labels;
        seg.segment(cloud, labels);
        expect(labels.empty(), "empty cloud gives no labels");
        std::printf("device\n");
    }
    catch (const std::runtime_error& e)
    {
        std::printf("nodevice %s\n", e.what());
    }
    return bad;
}
"""


def test_dropin_header_compiles_links_and_runs(built, tmp_path):
    src = tmp_path / "dropin.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(T.REPO, "include"),
                    "-I" + os.path.join(PKG, "cpp"), str(src), "-o", str(exe), "-L" + PKG, "-llp_gpu",
                    "-Wl,-rpath," + PKG], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    out = r.stdout.strip()
    assert out == "device" or out.startswith("nodevice "), out
