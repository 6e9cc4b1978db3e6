// lp_wire.cu — wire-format ingestion: a sensor_msgs/PointCloud2 byte buffer unpacked on the device
// into the library's XYZI (+ ring) arrays, as Processor's convert<PointT> does on the host
// (processor.cpp:42-179: float32 x, y, z and intensity, uint16 ring, each at its field offset within
// row * row_step + col * point_step).
#include "lidar_gb300.h"
#include "lp_common.cuh"
#include "lp_stages.hpp"

namespace lpg
{
namespace
{
// Little-endian reads byte by byte: fields need not be aligned (any point_step).
__device__ __forceinline__ float rd_f32(const uint8_t* p)
{
    const uint32_t u = static_cast<uint32_t>(p[0]) | (static_cast<uint32_t>(p[1]) << 8) |
                       (static_cast<uint32_t>(p[2]) << 16) | (static_cast<uint32_t>(p[3]) << 24);
    return __uint_as_float(u);
}

__global__ void k_unpack_pc2(const uint8_t* data, uint32_t width, uint32_t n, uint32_t point_step, uint32_t row_step,
                             uint4 off, uint32_t off_ring, float4* xyzi, uint16_t* ring)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const uint32_t row = i / width, col = i - row * width;
    const uint8_t* p = data + static_cast<size_t>(row) * row_step + static_cast<size_t>(col) * point_step;
    xyzi[i] = make_float4(rd_f32(p + off.x), rd_f32(p + off.y), rd_f32(p + off.z),
                          off.w != LP_NO_FIELD ? rd_f32(p + off.w) : 0.0f);
    if (ring && off_ring != LP_NO_FIELD)
        ring[i] = static_cast<uint16_t>(p[off_ring] | (p[off_ring + 1] << 8));
}
} // namespace

void launch_unpack_pointcloud2(cudaStream_t st, const uint8_t* data, uint32_t width, uint32_t height,
                               uint32_t point_step, uint32_t row_step, const uint32_t* offsets, float4* xyzi,
                               uint16_t* ring, uint64_t& launches)
{
    const uint32_t n = width * height;
    if (n == 0)
        return;
    k_unpack_pc2<<<div_up(n, 256u), 256, 0, st>>>(data, width, n, point_step, row_step,
                                                  make_uint4(offsets[0], offsets[1], offsets[2], offsets[3]), offsets[4],
                                                  xyzi, ring);
    launches += 1;
}
} // namespace lpg
