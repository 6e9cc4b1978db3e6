// Stand-in for the few PCL point structs the reference library names.
// Test infrastructure only: lets the reference's own .cpp files compile without PCL
// so that they can serve as the parity oracle. Only the members the reference reads exist.
#pragma once
#include <cstdint>
// PCL pulls Eigen in through its point types; the reference segmenter relies on that.
#include <Eigen/Dense>

#ifndef EIGEN_ALIGN16
#define EIGEN_ALIGN16 alignas(16)
#endif
#define PCL_ADD_POINT4D \
    float x;            \
    float y;            \
    float z;            \
    float data_pad_
#define EIGEN_MAKE_ALIGNED_OPERATOR_NEW
#define POINT_CLOUD_REGISTER_POINT_STRUCT(...)

namespace pcl
{
struct alignas(16) PointXYZ
{
    float x{0}, y{0}, z{0}, pad_{1};
    PointXYZ() = default;
    PointXYZ(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};

struct alignas(16) PointXYZI
{
    float x{0}, y{0}, z{0}, pad_{1};
    float intensity{0};
    PointXYZI() = default;
    PointXYZI(float x_, float y_, float z_, float i_) : x(x_), y(y_), z(z_), intensity(i_) {}
};

struct alignas(16) PointXYZRGB
{
    float x{0}, y{0}, z{0}, pad_{1};
    std::uint8_t b{0}, g{0}, r{0}, a{255};
    PointXYZRGB() = default;
    PointXYZRGB(float x_, float y_, float z_, std::uint8_t r_, std::uint8_t g_, std::uint8_t b_)
        : x(x_), y(y_), z(z_), b(b_), g(g_), r(r_)
    {
    }
};
} // namespace pcl
