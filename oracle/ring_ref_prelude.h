// Declarations that let the reference's Dataloader::addRingInfo (src/dataloader/src/dataloader.cpp:68-137)
// compile on its own, without ROS: oracle/build_ref.sh extracts that one function from the
// reference tree into oracle/_ref/add_ring_info.cpp, which includes this header first and
// ring_ref_capi.inc last. Test infrastructure only (pins the oracle's ring restatement).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>

#include <pcl/point_cloud.h>
#include <pcl/point_types.h>

#include "lidar_processing_lib/point_types.hpp"

namespace dataloading
{
// only the member the extracted function defines; the ROS node around it is not needed
struct Dataloader
{
    static void addRingInfo(const pcl::PointCloud<pcl::PointXYZI>& cloud_in, pcl::PointCloud<pcl::PointXYZIR>& cloud_out);
};
} // namespace dataloading
