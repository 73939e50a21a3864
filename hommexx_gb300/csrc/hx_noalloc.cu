// hx_noalloc.cu — DSS of a caller-owned device field without any device allocation.
//
// Some callers cannot allocate device memory when they need the operation: a host
// model that reserves its whole GPU memory budget at start-up and forbids allocations
// afterwards, or code that runs where cudaMalloc is not permitted.  For them,
// hx_dss_noalloc performs the same direct-stiffness summation as hx_run_dss (the
// gather in the reference's fixed accumulation order, optionally times rspheremp),
// but its scratch lives in a file-scope __device__ array of fixed size, HX_NOALLOC_MAX
// doubles (4 MiB).  The caller passes the input and output fields (device pointers,
// the output may alias the input); the connectivity and rspheremp come from the
// initialised session.
//
// When the array becomes device memory: CUDA loads a module (this file's kernels and
// its __device__ array) lazily by default, at the first use of one of its symbols.  So
// the set-up below runs during session initialisation (init_boundary_exchanges_c),
// while the host still allows allocation: it looks the array's address up on the
// session's device and queries both kernels, which loads the module and reserves the
// 4 MiB there.  From then on the device holds the array until the process exits, and
// hx_dss_noalloc itself loads, allocates and frees nothing.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/hxgpu.h"
#include "hx_common.h"

namespace hx {
bool session_dss_view(int* E, const int** cnt, const int** src, const double** rsp, cudaStream_t* s, int* dev);
}

namespace {

constexpr long long HX_NOALLOC_MAX = 1LL << 19;  // doubles: 4 MiB, up to 455 elements

static __device__ __align__(256) double g_noalloc_scratch[HX_NOALLOC_MAX];

// Device address of g_noalloc_scratch per device ordinal, looked up once with that
// device current; written and read under g_addr_mutex.
constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_addr_mutex;

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

namespace hx {

// Set-up of the no-allocation DSS on device `dev` (the session's): once per device, with
// that device current, the array's address is looked up and the kernels' attributes
// queried, which loads this module there.  The caller's current device is restored.
// Returns cudaSuccess or the first error.
cudaError_t noalloc_setup(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_addr_mutex);
  if (g_scratch_addr[dev]) return cudaSuccess;
  int prev = 0;
  cudaError_t e = cudaGetDevice(&prev);
  if (e != cudaSuccess) return e;
  if (prev != dev && (e = cudaSetDevice(dev)) != cudaSuccess) return e;
  void* p = nullptr;
  cudaFuncAttributes fa;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_noalloc_copy);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, k_noalloc_gather);
  if (e == cudaSuccess && !p) e = cudaErrorInvalidSymbol;
  if (e == cudaSuccess) g_scratch_addr[dev] = p;
  if (prev != dev) {
    const cudaError_t e2 = cudaSetDevice(prev);
    if (e == cudaSuccess) e = e2;
  }
  return e;
}

}  // namespace hx

extern "C" int hx_dss_noalloc(const double* in, double* out, int nelem, int apply_rspheremp) {
  char msg[256];
  int E = 0, sdev = -1;
  const int *cnt = nullptr, *src = nullptr;
  const double* rsp = nullptr;
  cudaStream_t stream = nullptr;
  if (!hx::session_dss_view(&E, &cnt, &src, &rsp, &stream, &sdev)) {
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
  // The session's tables and stream live on the session's device: the call must be made
  // with that device current.
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return HX_ERR_CUDA;
  if (dev != sdev) {
    std::fprintf(stderr, "hx_dss_noalloc: device %d is current, the session runs on device %d\n", dev, sdev);
    return HX_ERR_STATE;
  }
  double* scr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_addr_mutex);
    if (dev >= 0 && dev < kMaxDevices) scr = static_cast<double*>(g_scratch_addr[dev]);
  }
  if (!scr) {
    std::fprintf(stderr, "hx_dss_noalloc: no scratch on device %d (session set-up did not run there)\n", dev);
    return HX_ERR_STATE;
  }
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
