// Particle binning (get_particles_id_in_every_cell, 3D/run_3D.py:342-351) for callers that
// cannot allocate device memory: no handle, no workspace, no cudaMalloc.  Its scratch is one
// fixed array in the library's own device image, sized for PFM_NOALLOC_MAX_PARTICLES particles
// and PFM_NOALLOC_MAX_CELLS cells.  The result equals pfm3_sort_particles / pfm2_sort_particles
// bit for bit: counts by int(pos/dx) clamped to the grid, each bin in ascending particle index.
#include <mutex>

#include "pfm_binsort.cuh"
#include "pfm_internal.cuh"

namespace pfm {
namespace {

constexpr int kNaThreads = 256;
constexpr int kNaScanThreads = 1024;
constexpr int64_t kNaMaxP = PFM_NOALLOC_MAX_PARTICLES;
constexpr int64_t kNaMaxC = PFM_NOALLOC_MAX_CELLS;
// scratch layout (int32): slot[kNaMaxP] | start[kNaMaxC + 1] (padded to 64 entries)
constexpr int64_t kNaStartOff = kNaMaxP;
constexpr int64_t kNaWords = kNaMaxP + kNaMaxC + 64;
constexpr int kNaMaxDevices = 64;

// Shared by every call on a device: holds the previous call's slots and bin starts.
static __device__ __align__(256) int g_noalloc_scratch[kNaWords];

struct NaGrid {
  int N[3];
  float dx;
};

template <int D>
__device__ __forceinline__ int na_key(const float* __restrict__ pos, int64_t P, int64_t q, const NaGrid& g) {
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    int ci = __float2int_rz(pos[a * P + q] / g.dx);  // int(particles_pos[i] / dx)
    c[a] = ci < 0 ? 0 : (ci > g.N[a] - 1 ? g.N[a] - 1 : ci);
  }
  return (D == 3) ? (c[0] * g.N[1] + c[1]) * g.N[2] + c[2] : c[0] * g.N[1] + c[1];
}

__global__ void __launch_bounds__(kNaThreads) k_na_zero(int* __restrict__ a, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = 0;
}

template <int D>
__global__ void __launch_bounds__(kNaThreads) k_na_bin(const float* __restrict__ pos, int64_t P, NaGrid g,
                                                       int* __restrict__ slot, int* __restrict__ count) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  slot[q] = atomicAdd(&count[na_key<D>(pos, P, q, g)], 1);
}

// one block: start[c] = sum of count[0..c), start[C] = P.  Thread t owns a contiguous run.
__global__ void __launch_bounds__(kNaScanThreads) k_na_scan(const int* __restrict__ count, int64_t C,
                                                            int* __restrict__ start) {
  __shared__ int warp_tot[kNaScanThreads / 32];
  const int64_t run = (C + kNaScanThreads - 1) / kNaScanThreads;
  const int64_t b = threadIdx.x * run;
  const int64_t e = b + run < C ? b + run : C;
  int sum = 0;
  for (int64_t i = b; i < e; ++i) sum += count[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) warp_tot[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = warp_tot[lane];
    int wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += v;
    }
    warp_tot[lane] = wi - w;  // exclusive prefix of the warp totals
  }
  __syncthreads();
  int ex = warp_tot[warp] + incl - sum;
  for (int64_t i = b; i < e; ++i) {
    start[i] = ex;
    ex += count[i];
  }
  if (threadIdx.x == kNaScanThreads - 1) start[C] = ex;
}

template <int D>
__global__ void __launch_bounds__(kNaThreads) k_na_scatter(const float* __restrict__ pos, int64_t P, NaGrid g,
                                                           const int* __restrict__ slot,
                                                           const int* __restrict__ start, int* __restrict__ order) {
  int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= P) return;
  order[start[na_key<D>(pos, P, q, g)] + slot[q]] = (int)q;
}

// each bin in ascending particle index: bins of up to kSmallBin entries one thread each, larger
// ones by a whole block in k_bin_sort_big (pfm_binsort.cuh), so a bin holding every particle takes
// O(n log^2 n) work spread over a block instead of O(n^2) dependent steps
__global__ void __launch_bounds__(kNaThreads) k_na_cell_sort(const int* __restrict__ start, int64_t C,
                                                             int* __restrict__ order) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const int b = start[c], e = start[c + 1];
  sort_bin_by_thread(order, b, e - b);
}

// Device address of g_noalloc_scratch for the current device, looked up once per device and kept
// for the life of the process.  A cudaDeviceReset() ends the context that address belongs to: a
// process that resets a device must not call this entry point on that device afterwards.
int scratch_for_current_device(int** out) {
  static std::mutex mu;
  static int* addr[kNaMaxDevices] = {};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return PFM_ERR_CUDA;
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return PFM_ERR_CUDA;
    addr[dev] = static_cast<int*>(p);
  }
  *out = addr[dev];
  return PFM_OK;
}

inline unsigned blocks_for(int64_t n) { return (unsigned)((n + kNaThreads - 1) / kNaThreads); }

}  // namespace
}  // namespace pfm

using namespace pfm;

extern "C" int pfm_sort_particles_noalloc(int dim, const int res[3], double dx, int64_t particles,
                                          const float* pos, int* cell_count, int* order, void* stream) {
  if (dim != 2 && dim != 3) return PFM_ERR_ARG;
  if (!res || !cell_count) return PFM_ERR_NULL;
  if (particles < 0 || !(dx > 0.0)) return PFM_ERR_ARG;
  if (particles > 0 && (!pos || !order)) return PFM_ERR_NULL;
  NaGrid g{{1, 1, 1}, (float)dx};
  int64_t C = 1;
  for (int a = 0; a < dim; ++a) {
    if (res[a] < 1) return PFM_ERR_SHAPE;
    g.N[a] = res[a];
    C *= res[a];
    if (C > kNaMaxC) return PFM_ERR_SHAPE;
  }
  if (particles > kNaMaxP) return PFM_ERR_SHAPE;
  int* scratch = nullptr;
  if (scratch_for_current_device(&scratch)) return PFM_ERR_CUDA;
  int* slot = scratch;
  int* start = scratch + kNaStartOff;
  const int64_t P = particles;
  cudaStream_t st = (cudaStream_t)stream;
  k_na_zero<<<blocks_for(C), kNaThreads, 0, st>>>(cell_count, C);
  if (P > 0) {
    if (dim == 3)
      k_na_bin<3><<<blocks_for(P), kNaThreads, 0, st>>>(pos, P, g, slot, cell_count);
    else
      k_na_bin<2><<<blocks_for(P), kNaThreads, 0, st>>>(pos, P, g, slot, cell_count);
  }
  k_na_scan<<<1, kNaScanThreads, 0, st>>>(cell_count, C, start);
  if (P > 0) {
    if (dim == 3)
      k_na_scatter<3><<<blocks_for(P), kNaThreads, 0, st>>>(pos, P, g, slot, start, order);
    else
      k_na_scatter<2><<<blocks_for(P), kNaThreads, 0, st>>>(pos, P, g, slot, start, order);
    k_na_cell_sort<<<blocks_for(C), kNaThreads, 0, st>>>(start, C, order);
    k_bin_sort_big<<<(unsigned)((C + kBigThreads - 1) / kBigThreads), kBigThreads, 0, st>>>(start, C, order);
  }
  return cudaGetLastError() == cudaSuccess ? PFM_OK : PFM_ERR_CUDA;
}
