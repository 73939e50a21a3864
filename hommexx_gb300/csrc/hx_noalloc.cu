// hx_noalloc.cu — DSS of a caller-owned device field without any device allocation.
//
// Some callers cannot allocate device memory when they need the operation: a host
// model that reserves its whole GPU memory budget at start-up and forbids allocations
// afterwards, or code that runs where cudaMalloc is not permitted.  For them,
// hx_dss_noalloc performs the same direct-stiffness summation as hx_run_dss (the
// gather in the reference's fixed accumulation order, optionally times rspheremp),
// but its scratch lives in a file-scope __device__ array of fixed size, HX_NOALLOC_MAX
// doubles (4 MiB), reserved on every GPU that loads this library until the process
// exits.  The caller passes the input and output fields (device pointers, the output
// may alias the input); the connectivity and rspheremp come from the initialised
// session.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/hxgpu.h"
#include "hx_common.h"

namespace hx {
bool session_dss_view(int* E, const int** cnt, const int** src, const double** rsp, cudaStream_t* s);
}

namespace {

constexpr long long HX_NOALLOC_MAX = 1LL << 19;  // doubles: 4 MiB, up to 455 elements

static __device__ __align__(256) double g_noalloc_scratch[HX_NOALLOC_MAX];

// Device address of g_noalloc_scratch per device, looked up once with that device current.
void* g_scratch_addr[64] = {};

__global__ void k_noalloc_copy(const double* __restrict__ in, double* scr, long long n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) scr[i] = in[i];
}

__global__ void k_noalloc_gather(const double* __restrict__ scr, double* out, int E,
                                 const int* __restrict__ cnt, const int* __restrict__ src,
                                 const double* __restrict__ rsp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (long long)E * hx::NLEV * 16) return;
  const int e = (int)(i / (hx::NLEV * 16)), l = (int)((i / 16) % hx::NLEV), p = (int)(i & 15);
  const int ep = e * 16 + p;
  double acc = scr[i];
  const int n = cnt[ep];
  for (int k = 0; k < n; ++k) {
    const int s = src[ep * hx::MAXSRC + k];
    acc += scr[((long long)(s >> 4) * hx::NLEV + l) * 16 + (s & 15)];
  }
  if (rsp) acc *= rsp[ep];
  out[i] = acc;
}

}  // namespace

extern "C" int hx_dss_noalloc(const double* in, double* out, int nelem, int apply_rspheremp) {
  char msg[256];
  int E = 0;
  const int *cnt = nullptr, *src = nullptr;
  const double* rsp = nullptr;
  cudaStream_t stream = nullptr;
  if (!hx::session_dss_view(&E, &cnt, &src, &rsp, &stream)) {
    std::fprintf(stderr, "hx_dss_noalloc: the session is not initialised (init_boundary_exchanges_c)\n");
    return HX_ERR_STATE;
  }
  const long long n = (long long)nelem * hx::NLEV * 16;
  if (nelem != E || n <= 0) {
    std::snprintf(msg, sizeof msg, "hx_dss_noalloc: nelem=%d does not match the session's %d elements", nelem, E);
    std::fprintf(stderr, "%s\n", msg);
    return 13;
  }
  if (n > HX_NOALLOC_MAX) {
    std::snprintf(msg, sizeof msg,
                  "hx_dss_noalloc: %lld values exceed the fixed scratch of %lld doubles "
                  "(at most %lld elements of 72 levels)",
                  n, HX_NOALLOC_MAX, HX_NOALLOC_MAX / (hx::NLEV * 16));
    std::fprintf(stderr, "%s\n", msg);
    return 13;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return HX_ERR_CUDA;
  if (!g_scratch_addr[dev]) {
    // Set-up on the first call on this device, with the device current.
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      std::fprintf(stderr, "hx_dss_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
      return HX_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  double* scr = static_cast<double*>(g_scratch_addr[dev]);
  const unsigned blocks = (unsigned)((n + 255) / 256);
  k_noalloc_copy<<<blocks, 256, 0, stream>>>(in, scr, n);
  k_noalloc_gather<<<blocks, 256, 0, stream>>>(scr, out, E, cnt, src, apply_rspheremp ? rsp : nullptr);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    std::fprintf(stderr, "hx_dss_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return HX_ERR_CUDA;
  }
  return 0;
}
