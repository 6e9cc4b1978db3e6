// Stand-in for pcl::PointCloud<T>: a std::vector of points with the accessors the
// reference library uses. Test infrastructure only.
#pragma once
#include <cstddef>
#include <utility>
#include <vector>

namespace pcl
{
template <typename PointT>
struct PointCloud
{
    std::vector<PointT> points;

    std::size_t size() const noexcept { return points.size(); }
    bool empty() const noexcept { return points.empty(); }
    void clear() noexcept { points.clear(); }
    void reserve(std::size_t n) { points.reserve(n); }
    void push_back(const PointT& p) { points.push_back(p); }
    template <typename... Args>
    void emplace_back(Args&&... args)
    {
        points.emplace_back(std::forward<Args>(args)...);
    }
    const PointT& operator[](std::size_t i) const { return points[i]; }
    PointT& operator[](std::size_t i) { return points[i]; }
};
} // namespace pcl
