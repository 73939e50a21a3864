// hx_common.h — constants and argument structs shared by the kernels and the host
// runtime of libhxgpu.so.
//
// Device layout: exactly the Fortran layout the C ABI receives, so init/push are plain
// copies.  Per element and time level a 3-D scalar is [lev][16] and a 2-vector
// [lev][2][16]; the point index is p = igp*4 + jgp with the reference C++ names
// (igp = Fortran j, jgp = Fortran i).  Metric arrays are [E][2][2][16] (D, Dinv,
// metinv, tensorvisc), [E][2][3][16] (vec_sph2cart) and [E][16].
#pragma once
#include <cstddef>
#include <cstdint>

namespace hx {

constexpr int NP = 4;
constexpr int NP2 = 16;
constexpr int NLEV = 72;
constexpr int NTL = 3;
constexpr int QTL = 2;
constexpr int MAXSRC = 3;   // DSS contributions per point besides its own value

// src/share/cxx/PhysicalConstants.hpp:17-22
constexpr double kRwaterVapor = 461.5;
constexpr double kRgas = 287.04;
constexpr double kCp = 1005.0;
constexpr double kKappa = kRgas / kCp;
constexpr double kRrearth = 1.0 / 6.376e6;

template <typename R>
struct MetricP {
  const R* D;          // [E][2][2][16]
  const R* Dinv;
  const R* metinv;
  const R* metdet;     // [E][16]
  const R* spheremp;
  const R* rspheremp;
  const R* mp;
  const R* fcor;
  const R* phis;
  const R* tensorvisc;     // [E][2][2][16] or null
  const R* vec_sph2cart;   // [E][2][3][16] or null
  const double* spheremp_d;   // double copies for the state updates and the DSS
  const double* rspheremp_d;
  const double* lapm;  // FP64 form: weak Laplacian per element, [E][16 rows][16 cols]
};

// DSS gather table: for (e, p) the ordered sources src[(e*16+p)*3 + k] = se*16 + sp,
// k < cnt[e*16+p], in the reference accumulation order.  npts = E*16 and flag (the
// session's bounds-violation word) serve the index checks of the HX_BOUNDS_CHECK build.
struct DssTable {
  const int* cnt;
  const int* src;
  int npts;
  int* flag;
};

// Codes of the HX_BOUNDS_CHECK build's index checks, recorded in the flag word (the first
// violation wins) while the offending access is skipped.
enum BoundsCode : int {
  kBoundsDssPoint = 1,    // a gather for a point outside the table
  kBoundsDssCount = 2,    // more than MAXSRC (or a negative number of) contributions
  kBoundsDssSource = 3,   // a source index outside the mesh
  kBoundsRemapCell = 4,   // a remap source cell (kid) outside the column
  kBoundsTracerSlab = 5,  // a Qdp slab (tracer, time level) outside the array
};

// A 3-D field view: element e, level l, point p at base[e*es + l*ls + p].
template <typename T>
struct FieldV {
  T* base;
  long long es;
  int ls;
};

}  // namespace hx
