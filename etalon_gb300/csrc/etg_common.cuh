// Shared helpers of the etalon_gb300 CUDA sources: error reporting, IEEE-exact arithmetic,
// vector access and launch bookkeeping.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/etalon_gb300.h"

namespace etg {

void set_error(const char* fmt, ...);
int fault_injected(const char* where);  // host-side fault injection (ETG_FAULT)

#define ETG_TRY_CUDA(call)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) {                                                               \
      ::etg::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__,   \
                       __LINE__);                                                          \
      return ETG_ERR_CUDA;                                                                 \
    }                                                                                      \
  } while (0)

#define ETG_REQUIRE(cond, code, ...)   \
  do {                                 \
    if (!(cond)) {                     \
      ::etg::set_error(__VA_ARGS__);   \
      return (code);                   \
    }                                  \
  } while (0)

#define ETG_LAUNCH_CHECK() ETG_TRY_CUDA(cudaGetLastError())

// One IEEE rounding per operation and never a fused multiply-add, whatever the
// compiler flags: the reference rounds every NumPy ufunc result separately.
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }

// Counts kernel launches issued by the library (reported by the bench); engines on several
// host threads add to it concurrently.
extern std::atomic<int64_t> g_launches;

template <typename T>
struct Vec4;  // four consecutive elements, 16-byte (f32) or 2x16-byte (f64) accesses
template <>
struct Vec4<float> {
  float v[4];
  __device__ __forceinline__ void load(const float* p) {
    float4 a = *reinterpret_cast<const float4*>(p);
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  }
  __device__ __forceinline__ void store(float* p) const {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <>
struct Vec4<double> {
  double v[4];
  __device__ __forceinline__ void load(const double* p) {
    double2 a = reinterpret_cast<const double2*>(p)[0];
    double2 b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  __device__ __forceinline__ void store(double* p) const {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
  }
};

inline int dtype_ok(int dtype) { return dtype == ETG_F32 || dtype == ETG_F64; }

}  // namespace etg
