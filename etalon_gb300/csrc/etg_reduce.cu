// Device-side reductions for Etalon Studio's live view (etalon/studio/runner.py:258-291): the
// discrete field energy W = ½ ΔxΔy Σ (ε0 εr E² + μ0 Hz²) needs Σ f²/c over a field and its
// cb coefficient, and the snapshot needs block means of Hz. Both run on the device so a live
// run copies a few numbers or a small image, not the fields.
//
// Sums are float64 (float32 fields cannot overflow) and deterministic: fixed-size blocks
// write partial sums, one block adds the partials in order.
#include <algorithm>

#include "etg_common.cuh"

namespace etg {

constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 1024;

template <typename T>
__global__ void k_sum_sq(int64_t rows, int64_t cols, int64_t pitch, const T* __restrict__ f,
                         const T* __restrict__ c, double* __restrict__ partial) {
  __shared__ double sh[RED_THREADS];
  const int64_t n = rows * cols;
  double acc = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; q < n; q += (int64_t)gridDim.x * RED_THREADS) {
    const int64_t g = (q / cols) * pitch + q % cols;
    const double v = (double)f[g];
    acc += c ? v * v / (double)c[g] : v * v;
  }
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

__global__ void k_sum_partials(const double* __restrict__ partial, int n, double* __restrict__ out) {
  __shared__ double sh[RED_THREADS];
  double acc = 0.0;
  for (int q = threadIdx.x; q < n; q += RED_THREADS) acc += partial[q];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = RED_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// out[bi, bj] = mean of the sx x sy block at (bi*sx, bj*sy), accumulated in float64.
template <typename T, typename O>
__global__ void k_block_mean(int64_t mx, int64_t my, int sx, int sy, int64_t pitch, const T* __restrict__ f,
                             O* __restrict__ out) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= mx * my) return;
  const int64_t bi = q / my, bj = q % my;
  double acc = 0.0;
  for (int a = 0; a < sx; ++a)
    for (int b = 0; b < sy; ++b) acc += (double)f[(bi * sx + a) * pitch + bj * sy + b];
  out[q] = (O)(acc / ((double)sx * sy));
}

template <typename A, typename B>
__global__ void k_cast(int64_t n, const A* __restrict__ in, B* __restrict__ out) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    out[q] = (B)in[q];
}

}  // namespace etg

using namespace etg;

extern "C" {

int etg_sum_sq(int dtype, int64_t rows, int64_t cols, int64_t pitch, const void* field, const void* coeff,
               double* out) {
  ETG_REQUIRE(out && field && rows >= 0 && cols >= 0 && pitch >= cols, ETG_ERR_ARGUMENT, "etg_sum_sq: bad arguments");
  ETG_REQUIRE(dtype == ETG_F32 || dtype == ETG_F64, ETG_ERR_ARGUMENT, "etg_sum_sq: dtype must be 4 or 8");
  void* scratch = nullptr;  // partial sums, then the total
  int rc = etg_malloc(&scratch, (RED_BLOCKS + 1) * sizeof(double));
  if (rc) return rc;
  double* partial = (double*)scratch;
  const int64_t n = rows * cols;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(RED_BLOCKS, (n + RED_THREADS - 1) / RED_THREADS));
  if (dtype == ETG_F32)
    k_sum_sq<float><<<blocks, RED_THREADS>>>(rows, cols, pitch, (const float*)field, (const float*)coeff, partial);
  else
    k_sum_sq<double><<<blocks, RED_THREADS>>>(rows, cols, pitch, (const double*)field, (const double*)coeff, partial);
  k_sum_partials<<<1, RED_THREADS>>>(partial, blocks, partial + RED_BLOCKS);
  g_launches += 2;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, partial + RED_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(scratch);
  ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "etg_sum_sq: %s", cudaGetErrorString(e));
  return ETG_OK;
}

int etg_block_mean(int dtype, int64_t rows, int64_t cols, int64_t pitch, const void* field, int sx, int sy,
                   int out_dtype, void* out) {
  ETG_REQUIRE(field && out && sx > 0 && sy > 0 && pitch >= cols, ETG_ERR_ARGUMENT, "etg_block_mean: bad arguments");
  ETG_REQUIRE((dtype == ETG_F32 || dtype == ETG_F64) && (out_dtype == ETG_F32 || out_dtype == ETG_F64),
              ETG_ERR_ARGUMENT, "etg_block_mean: dtypes must be 4 or 8");
  const int64_t mx = rows / sx, my = cols / sy, n = mx * my;
  if (n == 0) return ETG_OK;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (dtype == ETG_F32 && out_dtype == ETG_F32)
    k_block_mean<float, float><<<grid, 256>>>(mx, my, sx, sy, pitch, (const float*)field, (float*)out);
  else if (dtype == ETG_F32)
    k_block_mean<float, double><<<grid, 256>>>(mx, my, sx, sy, pitch, (const float*)field, (double*)out);
  else if (out_dtype == ETG_F32)
    k_block_mean<double, float><<<grid, 256>>>(mx, my, sx, sy, pitch, (const double*)field, (float*)out);
  else
    k_block_mean<double, double><<<grid, 256>>>(mx, my, sx, sy, pitch, (const double*)field, (double*)out);
  g_launches += 1;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

int etg_cast(int from_dtype, int to_dtype, int64_t n, const void* in, void* out) {
  ETG_REQUIRE(in && out && n >= 0, ETG_ERR_ARGUMENT, "etg_cast: bad arguments");
  ETG_REQUIRE((from_dtype == ETG_F32 || from_dtype == ETG_F64) && (to_dtype == ETG_F32 || to_dtype == ETG_F64),
              ETG_ERR_ARGUMENT, "etg_cast: dtypes must be 4 or 8");
  if (n == 0) return ETG_OK;
  const unsigned grid = (unsigned)std::min<int64_t>(4096, (n + 255) / 256);
  if (from_dtype == to_dtype) {
    ETG_TRY_CUDA(cudaMemcpy(out, in, n * from_dtype, cudaMemcpyDeviceToDevice));
    return ETG_OK;
  }
  if (from_dtype == ETG_F32) k_cast<float, double><<<grid, 256>>>(n, (const float*)in, (double*)out);
  else k_cast<double, float><<<grid, 256>>>(n, (const double*)in, (float*)out);
  g_launches += 1;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

}  // extern "C"
