// mapmgr.cu — the map manager on the GPU (MapManager, mapManager.cpp:8-70;
// mapManager.h:7-10): the landmark map, its hit counts, the submap query
// and the update with a keyframe's cylinders and matches, all device
// resident, so that a keyframe sequence needs no host round trip for its
// map.
//
// getSubmap (mapManager.cpp:41-68): the k (100) nearest map roots to
// (x, y, 1) of the pose -- squared distances summed in double in x, y, z
// order and rounded to float, ties to the lower map index -- of which those
// among the `recent` (200) most recently added (map_size - index < recent,
// :60) form the submap, in distance order; the submap position of each
// remembers its map index.
// updateMap (mapManager.cpp:8-28): each cylinder in order; no match (-1)
// appends it with one hit; a match overwrites the matched map entry (the
// submap position's map index) and adds a hit.
#include "internal.h"
#include "scan_util.cuh"

namespace sg {
namespace {

constexpr int kMMThreads = 1024;

// Submap query, one block.  The rank of a recent entry j is the number of
// map entries before it in (distance, index) order; it is in the submap iff
// that rank is below k, and its submap position is the number of recent
// entries of lower rank.
__global__ void __launch_bounds__(kMMThreads) k_mm_submap(MapMgrDev m, double x, double y,
                                                        InPtrs* in) {
  __shared__ int sm[33];
  const int n = m.state[0];
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += blockDim.x) {
    const double dx = __dsub_rn(m.models[i].root[0], x), dy = __dsub_rn(m.models[i].root[1], y),
                 dz = __dsub_rn(m.models[i].root[2], 1.0);
    m.dist[i] = (float)__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
  }
  for (int s = tid; s < m.k; s += blockDim.x) m.slot[s] = -1;
  __syncthreads();
  const int j0 = max(0, n - m.recent + 1);
  for (int j = j0 + tid; j < n; j += blockDim.x) {
    const float dj = m.dist[j];
    int rank = 0;
    for (int i = 0; i < n; ++i) {
      const float di = m.dist[i];
      rank += (di < dj) || (di == dj && i < j);
    }
    if (rank < m.k) m.slot[rank] = j;
  }
  __syncthreads();
  int base = 0;
  for (int s0 = 0; s0 < m.k; s0 += blockDim.x) {
    const int s = s0 + tid;
    const int j = s < m.k ? m.slot[s] : -1;
    int total;
    const int ex = block_excl_scan(j >= 0 ? 1 : 0, sm, &total);
    if (j >= 0) {
      m.sub[base + ex] = m.models[j];
      m.sub_idx[base + ex] = j;
    }
    base += total;
  }
  if (tid == 0) {
    m.state[1] = base;
    if (in) {
      in->map = m.sub;
      in->n_map = base;
    }
  }
}

// Map update after a keyframe (one thread: later cylinders overwrite earlier
// ones in order, as the reference's loop does).  Runs when the keyframe's
// status is OK or not converged, and not for a later keyframe whose submap
// was empty (that keyframe is refused).
__global__ void k_mm_update(MapMgrDev m, Dev d, int first) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const Counters* c = d.cnt;
  const int status = first ? SLOAM_OK : c->status;
  if (!(status == SLOAM_OK || status == SLOAM_ERR_NOT_CONVERGED)) return;
  if (!first && m.state[1] == 0) return;
  int n = m.state[0];
  const int nsub = m.state[1];
  const int nc = c->n_cyl;
  for (int k = 0; k < nc; ++k) {
    const CylD& cy = d.cyls[k];
    sloam_cylinder o;
    for (int j = 0; j < 3; ++j) {
      o.root[j] = cy.root[j];
      o.ray[j] = cy.ray[j];
    }
    o.radius = cy.radius;
    o.id = cy.id;
    o.valid = 1;
    const int mt = first ? -1 : d.match_out[k];
    if (mt == -1) {
      if (n < m.cap) {
        m.models[n] = o;
        m.hits[n] = 1;
        ++n;
      } else {
        m.state[2] = 1;  // capacity exceeded
      }
    } else {
      const int idx = (mt >= 0 && mt < nsub) ? m.sub_idx[mt] : 0;
      m.models[idx] = o;
      m.hits[idx] += 1;
    }
  }
  m.state[0] = n;
}

}  // namespace

int launch_mm_submap(const MapMgrDev& m, double x, double y, InPtrs* d_in, cudaStream_t st) {
  k_mm_submap<<<1, kMMThreads, 0, st>>>(m, x, y, d_in);
  return 1;
}

int launch_mm_update(const MapMgrDev& m, const Dev& d, int first, cudaStream_t st) {
  k_mm_update<<<1, 32, 0, st>>>(m, d, first);
  return 1;
}

}  // namespace sg

// ------------------------------------------------------------------ C ABI
struct sloam_mapmgr {
  int device = 0;
  sg::MapMgrDev m{};
  void* mem = nullptr;
  cudaStream_t st = nullptr;
};

namespace {
template <typename T>
T* carve(unsigned char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += (n * sizeof(T) + 255) / 256 * 256;
  return r;
}
}  // namespace

extern "C" int sloam_mapmgr_create(int32_t device, int32_t capacity, int32_t k, int32_t recent,
                                   sloam_mapmgr** out) {
  if (!out || capacity < 1 || k < 1 || recent < 1) return SLOAM_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(device) != cudaSuccess) return SLOAM_ERR_CUDA;
  auto* mm = new sloam_mapmgr();
  mm->device = device;
  const size_t bytes = ((size_t)capacity * sizeof(sloam_cylinder) + 256) +
                       ((size_t)capacity * 4 + 256) * 2 + ((size_t)k * sizeof(sloam_cylinder) + 256) +
                       ((size_t)k * 4 + 256) * 2 + 256 * 2;
  if (cudaMalloc(&mm->mem, bytes) != cudaSuccess ||
      cudaStreamCreateWithFlags(&mm->st, cudaStreamNonBlocking) != cudaSuccess) {
    if (mm->mem) cudaFree(mm->mem);
    delete mm;
    return SLOAM_ERR_CUDA;
  }
  unsigned char* p = static_cast<unsigned char*>(mm->mem);
  sg::MapMgrDev& m = mm->m;
  m.cap = capacity;
  m.k = k;
  m.recent = recent;
  m.models = carve<sloam_cylinder>(p, capacity);
  m.hits = carve<int32_t>(p, capacity);
  m.dist = carve<float>(p, capacity);
  m.sub = carve<sloam_cylinder>(p, k);
  m.sub_idx = carve<int32_t>(p, k);
  m.slot = carve<int32_t>(p, k);
  m.state = carve<int32_t>(p, 4);
  if (cudaMemsetAsync(m.state, 0, 16, mm->st) != cudaSuccess ||
      cudaStreamSynchronize(mm->st) != cudaSuccess) {
    cudaFree(mm->mem);
    cudaStreamDestroy(mm->st);
    delete mm;
    return SLOAM_ERR_CUDA;
  }
  *out = mm;
  return SLOAM_OK;
}

extern "C" int sloam_mapmgr_destroy(sloam_mapmgr* mm) {
  if (!mm) return SLOAM_ERR_ARG;
  cudaSetDevice(mm->device);
  cudaStreamSynchronize(mm->st);
  cudaFree(mm->mem);
  cudaStreamDestroy(mm->st);
  delete mm;
  return SLOAM_OK;
}

extern "C" int sloam_mapmgr_size(sloam_mapmgr* mm, int32_t* n, int32_t* n_submap,
                                 int32_t* overflow) {
  if (!mm) return SLOAM_ERR_ARG;
  cudaSetDevice(mm->device);
  int32_t s[4];
  if (cudaMemcpy(s, mm->m.state, 16, cudaMemcpyDeviceToHost) != cudaSuccess) return SLOAM_ERR_CUDA;
  if (n) *n = s[0];
  if (n_submap) *n_submap = s[1];
  if (overflow) *overflow = s[2];
  return SLOAM_OK;
}

extern "C" int sloam_mapmgr_read(sloam_mapmgr* mm, sloam_cylinder* models, int32_t* hits,
                                 int32_t cap, int32_t* n) {
  if (!mm || cap < 0) return SLOAM_ERR_ARG;
  cudaSetDevice(mm->device);
  int32_t s[4];
  if (cudaMemcpy(s, mm->m.state, 16, cudaMemcpyDeviceToHost) != cudaSuccess) return SLOAM_ERR_CUDA;
  if (n) *n = s[0];
  const int c = s[0] < cap ? s[0] : cap;
  if (c > 0 && models &&
      cudaMemcpy(models, mm->m.models, sizeof(sloam_cylinder) * c, cudaMemcpyDeviceToHost) !=
          cudaSuccess)
    return SLOAM_ERR_CUDA;
  if (c > 0 && hits && cudaMemcpy(hits, mm->m.hits, 4 * (size_t)c, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SLOAM_ERR_CUDA;
  return s[0] > cap ? SLOAM_ERR_CAPACITY : SLOAM_OK;
}

extern "C" int sloam_mapmgr_load(sloam_mapmgr* mm, const sloam_cylinder* models,
                                 const int32_t* hits, int32_t n) {
  if (!mm || n < 0 || (n > 0 && (!models || !hits))) return SLOAM_ERR_ARG;
  if (n > mm->m.cap) return SLOAM_ERR_CAPACITY;
  cudaSetDevice(mm->device);
  const int32_t s[4] = {n, 0, 0, 0};
  if (n > 0 && (cudaMemcpy(mm->m.models, models, sizeof(sloam_cylinder) * n,
                           cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(mm->m.hits, hits, 4 * (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess))
    return SLOAM_ERR_CUDA;
  if (cudaMemcpy(mm->m.state, s, 16, cudaMemcpyHostToDevice) != cudaSuccess) return SLOAM_ERR_CUDA;
  return SLOAM_OK;
}

extern "C" int sloam_mapmgr_submap(sloam_mapmgr* mm, double x, double y, sloam_cylinder* out,
                                   int32_t* map_index, int32_t cap, int32_t* n_out) {
  if (!mm || cap < 0 || !n_out) return SLOAM_ERR_ARG;
  cudaSetDevice(mm->device);
  sg::launch_mm_submap(mm->m, x, y, nullptr, mm->st);
  if (cudaStreamSynchronize(mm->st) != cudaSuccess) return SLOAM_ERR_CUDA;
  int32_t s[4];
  if (cudaMemcpy(s, mm->m.state, 16, cudaMemcpyDeviceToHost) != cudaSuccess) return SLOAM_ERR_CUDA;
  *n_out = s[1];
  const int c = s[1] < cap ? s[1] : cap;
  if (c > 0 && out &&
      cudaMemcpy(out, mm->m.sub, sizeof(sloam_cylinder) * c, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SLOAM_ERR_CUDA;
  if (c > 0 && map_index &&
      cudaMemcpy(map_index, mm->m.sub_idx, 4 * (size_t)c, cudaMemcpyDeviceToHost) != cudaSuccess)
    return SLOAM_ERR_CUDA;
  return s[1] > cap ? SLOAM_ERR_CAPACITY : SLOAM_OK;
}

namespace sg {
const MapMgrDev& mapmgr_dev(const sloam_mapmgr* mm) { return mm->m; }
int mapmgr_device(const sloam_mapmgr* mm) { return mm->device; }
}  // namespace sg
