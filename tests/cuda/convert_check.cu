// Checks the integer-pipe double<->float conversions of hx_device.cuh against the
// hardware conversions, bit for bit: random bit patterns over every exponent, ties,
// zeros, subnormals, overflow, infinities and NaN; the Newton-Raphson reciprocal
// rcp_newton against IEEE division over positive divisors of exponents -120 .. 120, and
// the corrected quotient div_newton over numerators of exponents -300 .. 300 (both
// within one ulp), and the one-step rcp_newton1 (relative error below 2^-42).  Prints
// the mismatch counts; exit status 0 when there are none.
#include <cstdio>
#include <cstdlib>

#include "../../hommexx_gb300/csrc/hx_device.cuh"

namespace {

__device__ unsigned long long mix(unsigned long long x) {  // splitmix64 finaliser
  x += 0x9e3779b97f4a7c15ULL;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
  return x ^ (x >> 31);
}

__global__ void check(unsigned long long n, unsigned long long* bad) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long b = mix(i);
  const unsigned sel = (unsigned)(i & 7);
  if (sel == 1) b = (b & 0x800FFFFFE0000000ULL) | 0x10000000ULL | ((b >> 20) & 0x7FF0000000000000ULL);  // ties
  if (sel == 2) b &= 0x801FFFFFFFFFFFFFULL;   // tiny exponents (double/float subnormal range)
  if (sel == 3) b = (b & 0x800FFFFFFFFFFFFFULL) | ((unsigned long long)(1023 + (int)(b % 300) - 150) << 52);
  const double x = __longlong_as_double((long long)b);
  const float f1 = hx::d2f_rn(x), f2 = __double2float_rn(x);
  const unsigned u1 = __float_as_uint(f1), u2 = __float_as_uint(f2);
  const bool nan_ok = (f1 != f1) && (f2 != f2);
  if (u1 != u2 && !nan_ok) atomicAdd(bad, 1ULL);
  const float g = __uint_as_float((unsigned)mix(i ^ 0x5555ULL));
  const double d1 = hx::f2d(g), d2 = (double)g;
  const bool nan2 = (d1 != d1) && (d2 != d2);
  if (__double_as_longlong(d1) != __double_as_longlong(d2) && !nan2) atomicAdd(bad + 1, 1ULL);
  // reciprocal: positive x, exponent in [-120, 120]
  const unsigned long long m2 = mix(i ^ 0xABCDEFULL);
  const double x2 = __longlong_as_double((long long)((m2 & 0x000FFFFFFFFFFFFFULL) |
                                                     ((unsigned long long)(1023 - 120 + (int)((m2 >> 52) % 241)) << 52)));
  float rf;
  const long long r1 = __double_as_longlong(hx::rcp_newton(x2, rf)), r2 = __double_as_longlong(1.0 / x2);
  const long long du = r1 > r2 ? r1 - r2 : r2 - r1;
  if (du > 1) atomicAdd(bad + 2, 1ULL);
  if (du == 1) atomicAdd(bad + 3, 1ULL);
  // quotient: numerators of any sign over exponents -300 .. 300, the same divisors
  const unsigned long long m3 = mix(i ^ 0x13579BDFULL);
  const double a3 = __longlong_as_double((long long)((m3 & 0x800FFFFFFFFFFFFFULL) |
                                                     ((unsigned long long)(1023 - 300 + (int)((m3 >> 52) % 601)) << 52)));
  const long long q1 = __double_as_longlong(hx::div_newton(a3, x2, hx::rcp_newton(x2, rf)));
  const long long q2 = __double_as_longlong(a3 / x2);
  const long long dq = q1 > q2 ? q1 - q2 : q2 - q1;
  if (dq > 1) atomicAdd(bad + 4, 1ULL);
  if (dq == 1) atomicAdd(bad + 5, 1ULL);
  // one Newton step: relative error below 2^-42
  const double r1s = hx::rcp_newton1(x2, rf), r1e = 1.0 / x2;
  if (fabs(r1s - r1e) > 0x1p-42 * fabs(r1e)) atomicAdd(bad + 6, 1ULL);
}

}  // namespace

int main() {
  unsigned long long* bad = nullptr;
  if (cudaMalloc(&bad, 7 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  cudaMemset(bad, 0, 7 * sizeof(unsigned long long));
  const unsigned long long n = 1ULL << 26;
  check<<<(unsigned)((n + 255) / 256), 256>>>(n, bad);
  unsigned long long h[7] = {0, 0, 0, 0, 0, 0, 0};
  if (cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
  std::printf("d2f mismatches %llu, f2d mismatches %llu, rcp beyond 1 ulp %llu (1 ulp: %llu), "
              "div beyond 1 ulp %llu (1 ulp: %llu), one-step rcp beyond 2^-42 %llu, of %llu each\n", h[0], h[1],
              h[2], h[3], h[4], h[5], h[6], n);
  cudaFree(bad);
  return (h[0] == 0 && h[1] == 0 && h[2] == 0 && h[4] == 0 && h[6] == 0) ? 0 : 1;
}
