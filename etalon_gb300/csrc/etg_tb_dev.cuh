// Device-side pieces shared by the temporally blocked kernels (forward and adjoint).
#pragma once

#include "etg_sim.h"

namespace etg {

constexpr int TB_THREADS = 256;  // 8 warps of 32 lanes per tile

template <typename T>
struct TBVec;  // W elements per lane, one 16-byte access
template <>
struct TBVec<float> {
  static constexpr int W = 4;
  float v[4];
  __device__ __forceinline__ void ld(const float* p) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  }
  __device__ __forceinline__ void st(float* p) const {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
  __device__ __forceinline__ void zero() { v[0] = v[1] = v[2] = v[3] = 0.f; }
  __device__ __forceinline__ void fill(float x) { v[0] = v[1] = v[2] = v[3] = x; }
};
template <>
struct TBVec<double> {
  static constexpr int W = 2;
  double v[2];
  __device__ __forceinline__ void ld(const double* p) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    v[0] = a.x; v[1] = a.y;
  }
  __device__ __forceinline__ void st(double* p) const {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  }
  __device__ __forceinline__ void zero() { v[0] = v[1] = 0.0; }
  __device__ __forceinline__ void fill(double x) { v[0] = v[1] = x; }
};

template <typename T>
__device__ __forceinline__ T zero() { return T(0); }

// x is -0 (sign bit set, every other bit clear)
__device__ __forceinline__ bool is_neg_zero(float x) { return __float_as_uint(x) == 0x80000000u; }
__device__ __forceinline__ bool is_neg_zero(double x) {
  return __double_as_longlong(x) == (long long)0x8000000000000000ull;
}

// a compile-time bool carried as a value (for generic lambdas)
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};

}  // namespace etg
