// Checks the bulk asynchronous copy helpers of hx_device.cuh (bulk_load, mbar_wait):
// (1) a CTA streams slabs of 1152 doubles from global into one shared buffer, one slab
//     ahead, as the tracer loop of aal_tracer does, and writes back what it read: the
//     output equals the input bit for bit;
// (2) a wait on a barrier phase that never completes (nothing arrives) gives up after
//     its bounded number of polls and returns false; the kernel then exits normally and
//     the context stays usable (a later kernel runs and the host reads its result).
// Every access is in bounds and no copy is left in flight.  Exit status 0 on success.
#include <cstdio>
#include <vector>

#include "../../hommexx_gb300/csrc/hx_device.cuh"

namespace {

constexpr int SLAB = 72 * 16;  // doubles (9216 bytes)

__global__ void stream_slabs(const double* in, double* out, int nslab, int* fails) {
  __shared__ __align__(16) double buf[SLAB];
  __shared__ __align__(8) unsigned long long bar;
  const double* src = in + (size_t)blockIdx.x * nslab * SLAB;
  double* dst = out + (size_t)blockIdx.x * nslab * SLAB;
  if (threadIdx.x == 0) {
    hx::mbar_init(&bar, 1);
    hx::bulk_load(buf, src, SLAB * sizeof(double), &bar);
  }
  __syncthreads();
  unsigned parity = 0;
  for (int k = 0; k < nslab; ++k) {
    const bool ok = __syncthreads_and(hx::mbar_wait(&bar, parity, 1 << 20));
    parity ^= 1u;
    if (!ok) {
      if (threadIdx.x == 0) {
        atomicAdd(fails, 1);
        hx::mbar_wait(&bar, parity ^ 1u, 1 << 20);
      }
      return;
    }
    double v[SLAB / 128];
    for (int i = 0; i < SLAB / 128; ++i) v[i] = buf[threadIdx.x + 128 * i];
    __syncthreads();
    if (threadIdx.x == 0 && k + 1 < nslab) {
      hx::fence_proxy_async_smem();
      hx::bulk_load(buf, src + (size_t)(k + 1) * SLAB, SLAB * sizeof(double), &bar);
    }
    for (int i = 0; i < SLAB / 128; ++i) dst[(size_t)k * SLAB + threadIdx.x + 128 * i] = v[i];
  }
}

__global__ void wait_never(int* result) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) hx::mbar_init(&bar, 1);  // nothing will arrive
  __syncthreads();
  const bool ok = hx::mbar_wait(&bar, 0, 256);
  const bool any = __syncthreads_or(ok);
  if (threadIdx.x == 0) *result = any ? 1 : 2;
}

__global__ void add_one(int* x) { *x += 1; }

}  // namespace

int main() {
  const int blocks = 304, nslab = 10;
  const size_t n = (size_t)blocks * nslab * SLAB;
  std::vector<double> h(n), back(n);
  for (size_t i = 0; i < n; ++i) h[i] = (double)(i * 2654435761u % 1000003) * 1.0e-3 - 17.0;
  double *din = nullptr, *dout = nullptr;
  int *fails = nullptr, *res = nullptr;
  if (cudaMalloc(&din, n * 8) || cudaMalloc(&dout, n * 8) || cudaMalloc(&fails, 4) || cudaMalloc(&res, 4)) {
    std::printf("cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(din, h.data(), n * 8, cudaMemcpyHostToDevice);
  cudaMemset(dout, 0, n * 8);
  cudaMemset(fails, 0, 4);
  cudaMemset(res, 0, 4);
  stream_slabs<<<blocks, 128>>>(din, dout, nslab, fails);
  wait_never<<<1, 64>>>(res);
  add_one<<<1, 1>>>(res);
  const cudaError_t e = cudaDeviceSynchronize();
  int hf = -1, hr = -1;
  cudaMemcpy(back.data(), dout, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(&hf, fails, 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(&hr, res, 4, cudaMemcpyDeviceToHost);
  size_t bad = 0;
  for (size_t i = 0; i < n; ++i) bad += back[i] != h[i];
  std::printf("cuda %s, copied values wrong %zu of %zu, waits given up %d, timed-out wait result %d\n",
              cudaGetErrorString(e), bad, n, hf, hr);
  return (e == cudaSuccess && bad == 0 && hf == 0 && hr == 3) ? 0 : 1;
}
