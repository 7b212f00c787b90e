// noalloc.cu — projection + masking (a1/a2) for callers that cannot allocate
// device memory.
//
// Some callers of this library may not call cudaMalloc: plugins hosted by a
// process whose device-memory allocator owns the GPU (a pool that must not
// fragment, a real-time loop that forbids allocation after start-up, a
// sandbox whose budget was fixed at load).  sloam_project_mask_noalloc
// serves them: the caller passes its inputs and outputs, and every
// intermediate buffer of the projection kernels (pixel winner keys, pixel
// indices, range and mask images, the staged ground points, the column
// boundary table, the counters) lives in one file-scope __device__ array of
// kNoAllocBytes (about 4.2 MB, for at most kNoAllocMaxPoints = 131072 points
// and image widths up to 4096).  Every GPU that loads the library holds that
// array until the process exits.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr int kNoAllocMaxPoints = 131072;  // H * W at most (64 x 2048)
constexpr int kNoAllocMaxW = 4096;
constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffKey = 0;
constexpr size_t kOffPix = al(kOffKey + 8ull * kNoAllocMaxPoints);
constexpr size_t kOffRange = al(kOffPix + 4ull * kNoAllocMaxPoints);
constexpr size_t kOffMask = al(kOffRange + 4ull * kNoAllocMaxPoints);
constexpr size_t kOffGround = al(kOffMask + 1ull * kNoAllocMaxPoints);
constexpr size_t kOffBits = al(kOffGround + 16ull * kNoAllocMaxPoints);
constexpr size_t kOffBlk = al(kOffBits + 4ull * ((kNoAllocMaxPoints + 1023) / 1024 * 32 + 32));
constexpr size_t kOffTab = al(kOffBlk + 4ull * (kNoAllocMaxPoints / 256 + 64));
constexpr int kNoAllocMaxH = kNoAllocMaxPoints / 32;  // W >= 32
constexpr size_t kOffRowTab = al(kOffTab + 4ull * (kNoAllocMaxW + 1));
constexpr size_t kOffIn = al(kOffRowTab + 4ull * (kNoAllocMaxH + 1));
constexpr size_t kOffCnt = al(kOffIn + sizeof(sg::InPtrs));
constexpr size_t kNoAllocBytes = al(kOffCnt + sizeof(sg::Counters));

constexpr int kMaxContexts = 64;

}  // namespace

// The scratch of sloam_project_mask_noalloc.  Host code must not use this
// name as an address: the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

std::mutex g_mu;
// Device address of the scratch per CUDA context: a __device__ symbol has an
// address in each context that loads the module (the primary context of a
// device, or a context a plugin host created and made current itself).
struct ScratchAddr {
  void* cu_ctx;
  unsigned char* base;
};
ScratchAddr g_base[kMaxContexts] = {};
int g_nbase = 0;
using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn g_ctx_get = nullptr;
bool g_ctx_get_looked_up = false;
float g_tab[kNoAllocMaxW + 1];            // host staging of the column table
float g_row_tab[kNoAllocMaxH + 1];        // host staging of the row table

}  // namespace

extern "C" int sloam_project_mask_noalloc(const sloam_params* p, const float* d_xyzi, int32_t n,
                                          const uint8_t* d_point_labels,
                                          const uint8_t* d_mask_image, int32_t* d_pix,
                                          float* d_range_image, uint8_t* d_mask_out,
                                          int32_t* d_ground_idx, int32_t* d_n_ground,
                                          float* d_tree_cloud, void* stream) {
  if (!p || !d_xyzi || (!d_point_labels && !d_mask_image) || !d_ground_idx || !d_n_ground ||
      !d_tree_cloud)
    return SLOAM_ERR_ARG;
  if (p->img_w < 32 || p->img_h < 1 || (int64_t)p->img_w * p->img_h != n) return SLOAM_ERR_ARG;
  if (n > kNoAllocMaxPoints || p->img_w > kNoAllocMaxW) {
    std::fprintf(stderr,
                 "sloam_project_mask_noalloc: %d points / width %d exceed the fixed scratch "
                 "(at most %d points, width %d)\n",
                 n, p->img_w, kNoAllocMaxPoints, kNoAllocMaxW);
    return SLOAM_ERR_CAPACITY;
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    return SLOAM_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_ctx_get_looked_up) {
    g_ctx_get_looked_up = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_ctx_get = reinterpret_cast<CtxGetCurrentFn>(fn);
    cudaGetLastError();
  }
  // The runtime's current context for this device (its primary context
  // unless the caller made another one current).  The first call in a
  // context, made with that context current, looks the scratch's address
  // up; later calls in it reuse the address.
  void* cu_ctx = nullptr;
  if (!g_ctx_get || g_ctx_get(&cu_ctx) != 0 || !cu_ctx) {
    cudaGetLastError();
    cu_ctx = nullptr;  // unknown: look the address up on every call
  }
  unsigned char* b = nullptr;
  for (int i = 0; cu_ctx && i < g_nbase; ++i)
    if (g_base[i].cu_ctx == cu_ctx) b = g_base[i].base;
  if (!b) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) {
      cudaGetLastError();
      return SLOAM_ERR_CUDA;
    }
    b = static_cast<unsigned char*>(ptr);
    if (cu_ctx && g_nbase < kMaxContexts) g_base[g_nbase++] = ScratchAddr{cu_ctx, b};
  }
  sg::Dev d{};
  d.H = p->img_h;
  d.W = p->img_w;
  d.N = n;
  d.cap_ground = n;
  d.in = reinterpret_cast<sg::InPtrs*>(b + kOffIn);
  d.pkey = reinterpret_cast<unsigned long long*>(b + kOffKey);
  d.pix = reinterpret_cast<int32_t*>(b + kOffPix);
  d.range_img = reinterpret_cast<float*>(b + kOffRange);
  d.mask = reinterpret_cast<uint8_t*>(b + kOffMask);
  d.ground = reinterpret_cast<float4*>(b + kOffGround);
  d.gbits = reinterpret_cast<uint32_t*>(b + kOffBits);
  d.blk = reinterpret_cast<int32_t*>(b + kOffBlk);
  d.px_tab = reinterpret_cast<float*>(b + kOffTab);
  d.py_tab = reinterpret_cast<float*>(b + kOffRowTab);
  d.cnt = reinterpret_cast<sg::Counters*>(b + kOffCnt);
  d.tree = reinterpret_cast<float4*>(d_tree_cloud);
  d.ground_idx = d_ground_idx;
  const sg::KParams kp = sg::make_kparams(*p);
  // The previous call's contents remain: re-upload the tables and the input
  // pointers, and re-arm the pixel keys (they must start empty).
  sg::build_px_table(*p, g_tab);
  sg::build_py_table(*p, g_row_tab);
  sg::InPtrs in{};
  in.xyzi = reinterpret_cast<const float4*>(d_xyzi);
  in.plabel = d_point_labels;
  in.mask_in = d_mask_image;
  cudaError_t e = cudaMemcpyAsync(d.px_tab, g_tab, sizeof(float) * (p->img_w + 1),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d.py_tab, g_row_tab, sizeof(float) * (p->img_h + 1),
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d.in, &in, sizeof(in), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.pkey, 0xFF, sizeof(unsigned long long) * n, st);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SLOAM_ERR_CUDA;
  }
  sg::launch_begin(d, -1, 0, 0, 0, 0, st);
  sg::launch_project(d, kp, d_point_labels != nullptr, st);
  e = cudaMemcpyAsync(d_n_ground, &d.cnt->n_ground, sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && d_pix)
    e = cudaMemcpyAsync(d_pix, d.pix, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && d_range_image)
    e = cudaMemcpyAsync(d_range_image, d.range_img, 4 * (size_t)n, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && d_mask_out)
    e = cudaMemcpyAsync(d_mask_out, d.mask, (size_t)n, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaGetLastError();
    return SLOAM_ERR_CUDA;
  }
  return SLOAM_OK;
}
