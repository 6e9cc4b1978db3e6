// lp_split.cu — the processor's ground / obstacle / unsegmented clouds (processor.cpp:558-579) on
// the device: for each label class, one look-back scan over the labels whose epilogue writes every
// member point, in input order, as a coloured XYZRGB record at its exclusive prefix.
#include "lidar_gb300.h"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
// class 0: GROUND, 1: OBSTACLE, 2: any other label
__device__ __forceinline__ uint32_t in_class(uint32_t label, int cls)
{
    if (cls == 0)
        return label == LP_LABEL_GROUND;
    if (cls == 1)
        return label == LP_LABEL_OBSTACLE;
    return label != LP_LABEL_GROUND && label != LP_LABEL_OBSTACLE;
}

struct SplitSrc
{
    const uint32_t* lab;
    uint32_t n;
    int cls;
    __device__ __forceinline__ uint4 get4(uint32_t i) const
    {
        uint4 f;
        f.x = (i < n) ? in_class(lab[i], cls) : 0u;
        f.y = (i + 1u < n) ? in_class(lab[i + 1u], cls) : 0u;
        f.z = (i + 2u < n) ? in_class(lab[i + 2u], cls) : 0u;
        f.w = (i + 3u < n) ? in_class(lab[i + 3u], cls) : 0u;
        return f;
    }
};

// Writes member i at its exclusive prefix e; at i == n (the scan runs over n + 1 entries) e is the
// class's point count.
struct SplitDst
{
    const float4* pts;
    lp_xyzrgb* out;
    uint32_t n;
    uint32_t* count;
    uchar4 rgba;
    __device__ __forceinline__ void one(uint32_t i, uint32_t e, uint32_t f) const
    {
        if (i < n && f)
        {
            const float4 p = pts[i];
            lp_xyzrgb q;
            q.x = p.x;
            q.y = p.y;
            q.z = p.z;
            q.r = rgba.x;
            q.g = rgba.y;
            q.b = rgba.z;
            q.a = rgba.w;
            out[e] = q;
        }
        if (i == n)
            *count = e;
    }
    __device__ __forceinline__ void put4(uint32_t i, uint4 e, uint4 f) const
    {
        one(i, e.x, f.x);
        one(i + 1u, e.y, f.y);
        one(i + 2u, e.z, f.z);
        one(i + 3u, e.w, f.w);
    }
};
} // namespace

void launch_split_clouds(cudaStream_t st, const float4* pts, const uint32_t* labels, uint32_t n, lp_xyzrgb* out,
                         uint32_t* counts, uint32_t* sums, uint64_t& launches)
{
    // processor.cpp:568-578
    const uchar4 colour[3] = {make_uchar4(124, 252, 0, 255), make_uchar4(200, 0, 0, 255), make_uchar4(255, 255, 0, 255)};
    for (int c = 0; c < 3; ++c)
    {
        scan_lookback(st, SplitSrc{labels, n, c}, SplitDst{pts, out + static_cast<size_t>(c) * n, n, counts + c, colour[c]},
                      n + 1u, sums, nullptr);
        launches += 1;
    }
}
} // namespace lpg
