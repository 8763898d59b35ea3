// FP32 throughput probe: the denominator of the FP32 roofline that the particle and midpoint RK4
// kernels are reported against beside HBM bandwidth.  Each thread advances 8 independent FMA
// chains x <- x * a + b (|a| < 1, so the values stay bounded), with scalar FMAs or with packed
// f32x2 FMAs; the sum is stored only if it takes a value the chains cannot reach, which keeps the
// compiler from removing the work.
#include <cuda_runtime.h>

#include "../../include/pfm.h"

namespace pfm {

constexpr int kProbeThreads = 256;
constexpr int kChains = 8;

// PACKED: the 8 chains as 4 pairs advanced by packed f32x2 FMAs (__ffma2_rn), 2 FMAs per instruction
template <bool PACKED>
__global__ void __launch_bounds__(kProbeThreads) k_fma_rate(float* __restrict__ sink, int iters, float a, float b) {
  float s = 0.f;
  if (PACKED) {
    float2 x[kChains / 2];
    const float2 a2 = make_float2(a, a), b2 = make_float2(b, b);
#pragma unroll
    for (int c = 0; c < kChains / 2; ++c) x[c] = make_float2(1e-3f * (float)threadIdx.x + (float)c, (float)c + 0.5f);
#pragma unroll 4
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int c = 0; c < kChains / 2; ++c) x[c] = __ffma2_rn(x[c], a2, b2);
#pragma unroll
    for (int c = 0; c < kChains / 2; ++c) s += x[c].x + x[c].y;
  } else {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = 1e-3f * (float)threadIdx.x + (float)c;
#pragma unroll 4
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
#pragma unroll
    for (int c = 0; c < kChains; ++c) s += x[c];
  }
  if (s == -1.0f) sink[0] = s;  // the chains stay positive: never taken
}

}  // namespace pfm

extern "C" int pfm_measure_fp32_peak(float* sink, int blocks_per_sm, int iters, int reps, int packed, double* tflops,
                                     void* stream) {
  if (!tflops || !sink) return PFM_ERR_NULL;
  if (blocks_per_sm < 1 || blocks_per_sm > 64 || iters < 1 || reps < 1 || packed < 0 || packed > 1) return PFM_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return PFM_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const unsigned blocks = (unsigned)(sms * blocks_per_sm);
  double best = 0.0;
  int rc = PFM_OK;
  for (int r = 0; r < reps + 1 && rc == PFM_OK; ++r) {  // the first launch warms up
    cudaEventRecord(e0, st);
    if (packed)
      pfm::k_fma_rate<true><<<blocks, pfm::kProbeThreads, 0, st>>>(sink, iters, 0.9999999f, 1e-7f);
    else
      pfm::k_fma_rate<false><<<blocks, pfm::kProbeThreads, 0, st>>>(sink, iters, 0.9999999f, 1e-7f);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      rc = PFM_ERR_CUDA;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * pfm::kChains * (double)iters * blocks * pfm::kProbeThreads;
    const double rate = ms > 0.f ? flops / (ms * 1e-3) / 1e12 : 0.0;
    if (r > 0 && rate > best) best = rate;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *tflops = best;
  return rc;
}
