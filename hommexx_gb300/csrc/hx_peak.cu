// hx_peak.cu — measured FP64 roof of this GPU, for the roofline of the FP64 form.
//
// The FP64-form kernels are bound by the FP64 pipe rather than by HBM, so their
// roofline needs the FP64 rate this device sustains.  hx_fp64_peak measures it with a
// kernel of independent fused multiply-add chains (eight per thread, enough to cover
// the pipe latency at any occupancy), one wave of CTAs per SM at full occupancy, timed
// with CUDA events on a stream of its own after a warm-up launch.
#include <cuda_runtime.h>

#include "../../include/hxgpu.h"

namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_dfma_peak(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = 1e-3 * (threadIdx.x + c);
#pragma unroll 1
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == -1.0) out[0] = s;  // never true for these inputs; keeps the chains live
}

}  // namespace

extern "C" int hx_fp64_peak(double* tflops) {
  if (!tflops) return 13;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_dfma_peak, 256, 0) != cudaSuccess)
    return HX_ERR_CUDA;
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  const int iters = 1 << 14;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  double* out = nullptr;
  int rc = HX_ERR_CUDA;
  float ms = 0.f;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess && cudaEventCreate(&e0) == cudaSuccess &&
      cudaEventCreate(&e1) == cudaSuccess && cudaMalloc(&out, sizeof(double)) == cudaSuccess) {
    k_dfma_peak<<<blocks, 256, 0, st>>>(out, iters / 8, 0.999999, 1e-7);  // warm-up
    cudaEventRecord(e0, st);
    k_dfma_peak<<<blocks, 256, 0, st>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0.f) {
      const double flops = 2.0 * kChains * (double)iters * blocks * 256.0;
      *tflops = flops / (ms * 1e-3) / 1e12;
      rc = 0;
    }
  }
  if (out) cudaFree(out);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  return rc;
}
