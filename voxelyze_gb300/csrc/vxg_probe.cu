// Measured FP64 rate of this GPU, the denominator of the FP64 path's compute roofline.
//
// The FP64 time step is bound by the FP64 pipe, not by memory: every double add, multiply and
// fused multiply-add of the link and voxel passes issues there.  This probe keeps that pipe busy
// with independent fma.rn.f64 chains (eight per thread, 48 warps per SM) and times them with CUDA
// events; one FMA is two floating-point operations and one FP64 pipe instruction.
#include <cuda_runtime.h>

#include <algorithm>

#include "vxg.h"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 512;

__global__ void __launch_bounds__(kThreads) k_fp64_fma(double* out, int iters, double m, double c) {
  double a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) a[k] = 1e-3 * (threadIdx.x + 1) + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) asm volatile("fma.rn.f64 %0, %0, %1, %2;" : "+d"(a[k]) : "d"(m), "d"(c));
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += a[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains live; never true for these inputs
}

}  // namespace

extern "C" int vxg_probe_fp64_rate(int device, int iters, double* fma_per_s, float* ms) {
  if (!fma_per_s || iters <= 0) return VXG_E_ARG;
  *fma_per_s = 0;
  if (ms) *ms = 0;
  int prev = -1;
  if (cudaGetDevice(&prev) != cudaSuccess || cudaSetDevice(device) != cudaSuccess) return VXG_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fp64_fma, kThreads, 0);
  const int grid = std::max(1, sms * std::max(1, per_sm));
  double* d = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t st = nullptr;
  int rc = VXG_OK;
  float best = 0;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess || cudaEventCreate(&a) != cudaSuccess ||
      cudaEventCreate(&b) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
    rc = VXG_E_CUDA;
  } else {
    k_fp64_fma<<<grid, kThreads, 0, st>>>(d, std::max(1, iters / 16), 0.999999, 1e-9);  // warm-up
    for (int r = 0; r < 5 && rc == VXG_OK; ++r) {
      cudaEventRecord(a, st);
      k_fp64_fma<<<grid, kThreads, 0, st>>>(d, iters, 0.999999, 1e-9);
      cudaEventRecord(b, st);
      if (cudaEventSynchronize(b) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        rc = VXG_E_CUDA;
        break;
      }
      float t = 0;
      cudaEventElapsedTime(&t, a, b);
      if (best == 0 || t < best) best = t;
    }
  }
  if (rc == VXG_OK && best > 0) {
    *fma_per_s = (double)grid * kThreads * kChains * (double)iters / (best * 1e-3);
    if (ms) *ms = best;
  }
  if (st) cudaStreamDestroy(st);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (d) cudaFree(d);
  if (prev >= 0) cudaSetDevice(prev);
  return rc;
}
