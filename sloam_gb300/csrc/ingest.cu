// ingest.cu — input ingestion: points of a sensor message (the layout of a
// sensor_msgs/PointCloud2: fixed point_step bytes per point, little-endian
// fields at byte offsets) packed into the float4 XYZI array the keyframe
// path reads.  On the host the reference converts the message
// (pcl::fromROSMsg in InputManager::FindPC, inputNode.cpp:247) and packs
// XYZI again before the projection (Segmentation::run,
// inference.cpp:374-379); here it is one coalesced pass on the device.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sloam_gb300.h"

namespace {

__device__ __forceinline__ uint32_t load_u32(const unsigned char* p, bool aligned) {
  if (aligned) return *reinterpret_cast<const uint32_t*>(p);
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

__global__ void k_pack_points(const unsigned char* __restrict__ src, int n, int step, int ox,
                              int oy, int oz, int oi, int itype, float4* __restrict__ dst) {
  const bool aligned = ((step | ox | oy | oz | (oi < 0 ? 0 : oi)) & 3) == 0 &&
                       (reinterpret_cast<uintptr_t>(src) & 3) == 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned char* p = src + (size_t)i * step;
    float4 v;
    v.x = __uint_as_float(load_u32(p + ox, aligned));
    v.y = __uint_as_float(load_u32(p + oy, aligned));
    v.z = __uint_as_float(load_u32(p + oz, aligned));
    if (itype == SLOAM_FIELD_FLOAT32) v.w = __uint_as_float(load_u32(p + oi, aligned));
    else if (itype == SLOAM_FIELD_UINT16) v.w = (float)((uint32_t)p[oi] | ((uint32_t)p[oi + 1] << 8));
    else if (itype == SLOAM_FIELD_UINT8) v.w = (float)p[oi];
    else v.w = 0.0f;
    dst[i] = v;
  }
}

}  // namespace

extern "C" int sloam_pack_points(const void* d_points, int32_t n, int32_t point_step,
                                 int32_t off_x, int32_t off_y, int32_t off_z, int32_t off_i,
                                 int32_t intensity_type, float* d_xyzi, void* stream) {
  if (n < 0 || (n > 0 && (!d_points || !d_xyzi))) return SLOAM_ERR_ARG;
  if (intensity_type < SLOAM_FIELD_NONE || intensity_type > SLOAM_FIELD_UINT8) return SLOAM_ERR_ARG;
  const int isz = intensity_type == SLOAM_FIELD_FLOAT32 ? 4
                  : intensity_type == SLOAM_FIELD_UINT16 ? 2
                  : intensity_type == SLOAM_FIELD_UINT8  ? 1 : 0;
  for (int o : {off_x, off_y, off_z})
    if (o < 0 || o + 4 > point_step) return SLOAM_ERR_ARG;
  if (isz && (off_i < 0 || off_i + isz > point_step)) return SLOAM_ERR_ARG;
  if (n == 0) return SLOAM_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  k_pack_points<<<blocks, 256, 0, st>>>(static_cast<const unsigned char*>(d_points), n, point_step,
                                        off_x, off_y, off_z, isz ? off_i : -1, intensity_type,
                                        reinterpret_cast<float4*>(d_xyzi));
  return cudaGetLastError() == cudaSuccess ? SLOAM_OK : SLOAM_ERR_CUDA;
}
