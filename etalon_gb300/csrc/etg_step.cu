// Library basics (errors, device info, memory) and the per-step protocol kernels:
// one launch per method of Etalon's backend protocol, on arrays in TEState layout.
//
// The per-step kernels are what Etalon's unchanged FDTDSolver drives through the
// backend object (etalon/fdtd/solver.py:120-128). Each node's update performs the
// NumPy reference's operations in its order (numpy_backend.py:41-67) with explicitly
// rounded intrinsics, so results are bit-identical in float32 and float64.
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "etg_common.cuh"

namespace etg {

static thread_local std::string t_error;
std::atomic<int64_t> g_launches{0};

void set_error(const char* fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_error = buf;
}

// ETG_FAULT=<where> makes the named entry point fail with ETG_ERR_INJECTED before it
// touches the device; the host-side failure paths are tested this way.
int fault_injected(const char* where) {
  const char* f = getenv("ETG_FAULT");
  if (f && *f && (strcmp(f, where) == 0 || strcmp(f, "all") == 0)) {
    set_error("fault injected at %s (ETG_FAULT=%s)", where, f);
    return 1;
  }
  return 0;
}

// ---------------------------------------------------------------- per-step kernels

template <typename T>
__global__ void k_update_h(int nx, int ny, T* __restrict__ hz, const T* __restrict__ ex,
                           const T* __restrict__ ey, T* __restrict__ psx, T* __restrict__ psy,
                           const T* __restrict__ bxh, const T* __restrict__ cxh,
                           const T* __restrict__ ikxh, const T* __restrict__ byh,
                           const T* __restrict__ cyh, const T* __restrict__ ikyh, T db, T inv_dx,
                           T inv_dy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nx || j >= ny) return;
  const size_t k = (size_t)i * ny + j;          // Hz(i, j), Ey(i, j)
  const size_t kx = (size_t)i * (ny + 1) + j;   // Ex(i, j)
  const T dex_dy = mul(sub(ex[kx + 1], ex[kx]), inv_dy);
  const T dey_dx = mul(sub(ey[k + ny], ey[k]), inv_dx);
  const T py = add(mul(byh[j], psy[k]), mul(cyh[j], dex_dy));
  const T px = add(mul(bxh[i], psx[k]), mul(cxh[i], dey_dx));
  psy[k] = py;
  psx[k] = px;
  hz[k] = add(hz[k], mul(db, sub(add(mul(dex_dy, ikyh[j]), py), add(mul(dey_dx, ikxh[i]), px))));
}

template <typename T>
__global__ void k_update_e(int nx, int ny, T* __restrict__ ex, T* __restrict__ ey,
                           const T* __restrict__ hz, T* __restrict__ pey, T* __restrict__ pex,
                           const T* __restrict__ cbx, const T* __restrict__ cby,
                           const T* __restrict__ bxe, const T* __restrict__ cxe,
                           const T* __restrict__ ikxe, const T* __restrict__ bye,
                           const T* __restrict__ cye, const T* __restrict__ ikye, T inv_dx,
                           T inv_dy) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // over (nx + 1) x (ny + 1)
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i < nx && j >= 1 && j <= ny - 1) {  // Ex(i, j); j = 0 and j = ny are PEC
    const size_t k = (size_t)i * (ny + 1) + j;
    const size_t kh = (size_t)i * ny + j;
    const T d = mul(sub(hz[kh], hz[kh - 1]), inv_dy);
    const T p = add(mul(bye[j], pey[k]), mul(cye[j], d));
    pey[k] = p;
    ex[k] = add(ex[k], mul(cbx[k], add(mul(d, ikye[j]), p)));
  }
  if (i >= 1 && i <= nx - 1 && j < ny) {  // Ey(i, j); i = 0 and i = nx are PEC
    const size_t k = (size_t)i * ny + j;
    const T d = mul(sub(hz[k], hz[k - ny]), inv_dx);
    const T p = add(mul(bxe[i], pex[k]), mul(cxe[i], d));
    pex[k] = p;
    ey[k] = sub(ey[k], mul(cby[k], add(mul(d, ikxe[i]), p)));
  }
}

template <typename T>
__global__ void k_accumulate_dft(int n_f, int n_nodes, T* __restrict__ acc,
                                 const T* __restrict__ field, const int64_t* __restrict__ index,
                                 const T* __restrict__ ph) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int f = blockIdx.y;
  if (k >= n_nodes || f >= n_f) return;
  const T v = field[index[k]];
  const size_t a = 2 * ((size_t)f * n_nodes + k);
  // (v + 0i)(re + i im) = (v re, v im) exactly; then a complex add (numpy_backend.py:67)
  acc[a] = add(acc[a], mul(v, ph[2 * f]));
  acc[a + 1] = add(acc[a + 1], mul(v, ph[2 * f + 1]));
}

// NumPy `field[i, j] -= delta`: gather every value, subtract, then scatter in order,
// so duplicated nodes behave as in NumPy (last write wins). n is a handful of nodes.
template <typename T>
__global__ void k_scatter_sub(int64_t n_cols, int n, T* __restrict__ field,
                              const int64_t* __restrict__ ii, const int64_t* __restrict__ jj,
                              const T* __restrict__ delta) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  constexpr int CHUNK = 64;
  for (int base = 0; base < n; base += CHUNK) {
    T vals[CHUNK];
    const int m = min(CHUNK, n - base);
    for (int k = 0; k < m; ++k) vals[k] = sub(field[ii[base + k] * n_cols + jj[base + k]], delta[base + k]);
    for (int k = 0; k < m; ++k) field[ii[base + k] * n_cols + jj[base + k]] = vals[k];
  }
}

}  // namespace etg

using namespace etg;

// ---------------------------------------------------------------- C ABI

extern "C" {

const char* etg_last_error(void) { return t_error.c_str(); }

int etg_version(void) { return (1 << 16) | 0; }

int etg_device_info(int* device, char* name, int name_len, int* sm_count) {
  int dev = 0;
  ETG_TRY_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  ETG_TRY_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (device) *device = dev;
  if (name && name_len > 0) {
    strncpy(name, prop.name, name_len - 1);
    name[name_len - 1] = 0;
  }
  if (sm_count) *sm_count = prop.multiProcessorCount;
  return ETG_OK;
}

int etg_synchronize(void) {
  ETG_TRY_CUDA(cudaDeviceSynchronize());
  return ETG_OK;
}

int etg_set_device(int device) {
  ETG_TRY_CUDA(cudaSetDevice(device));
  return ETG_OK;
}

int etg_host_alloc(void** ptr, size_t bytes) {
  ETG_REQUIRE(ptr, ETG_ERR_ARGUMENT, "etg_host_alloc: null output pointer");
  *ptr = nullptr;
  cudaError_t e = cudaMallocHost(ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("etg_host_alloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    return ETG_ERR_ALLOC;
  }
  return ETG_OK;
}

int etg_host_free(void* ptr) {
  if (ptr) ETG_TRY_CUDA(cudaFreeHost(ptr));
  return ETG_OK;
}

int etg_malloc(void** ptr, size_t bytes) {
  ETG_REQUIRE(ptr, ETG_ERR_ARGUMENT, "etg_malloc: null output pointer");
  if (fault_injected("etg_malloc")) return ETG_ERR_INJECTED;
  *ptr = nullptr;
  cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error("etg_malloc(%zu bytes): %s", bytes, cudaGetErrorString(e));
    return ETG_ERR_ALLOC;
  }
  return ETG_OK;
}

int etg_free(void* ptr) {
  if (ptr) ETG_TRY_CUDA(cudaFree(ptr));
  return ETG_OK;
}

int etg_memcpy_h2d(void* dst, const void* src, size_t bytes) {
  if (bytes) ETG_TRY_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return ETG_OK;
}
int etg_memcpy_d2h(void* dst, const void* src, size_t bytes) {
  if (bytes) ETG_TRY_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return ETG_OK;
}
int etg_memcpy_d2d(void* dst, const void* src, size_t bytes) {
  if (bytes) ETG_TRY_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToDevice));
  return ETG_OK;
}
int etg_memset(void* dst, int value, size_t bytes) {
  if (bytes) ETG_TRY_CUDA(cudaMemset(dst, value, bytes));
  return ETG_OK;
}

int etg_update_h_te(int dtype, int nx, int ny, void* hz, const void* ex, const void* ey,
                    void* psi_hz_x, void* psi_hz_y, const void* bx_h, const void* cx_h,
                    const void* ikx_h, const void* by_h, const void* cy_h, const void* iky_h,
                    double db, double inv_dx, double inv_dy) {
  ETG_REQUIRE(dtype_ok(dtype) && nx > 0 && ny > 0 && nx <= 524272, ETG_ERR_ARGUMENT,  // rows of 8 on gridDim.y
              "etg_update_h_te: bad dtype %d or size %d x %d", dtype, nx, ny);
  if (fault_injected("etg_update_h_te")) return ETG_ERR_INJECTED;
  dim3 block(32, 8), grid((ny + 31) / 32, (nx + 7) / 8);
  if (dtype == ETG_F32) {
    k_update_h<float><<<grid, block>>>(nx, ny, (float*)hz, (const float*)ex, (const float*)ey,
        (float*)psi_hz_x, (float*)psi_hz_y, (const float*)bx_h, (const float*)cx_h,
        (const float*)ikx_h, (const float*)by_h, (const float*)cy_h, (const float*)iky_h,
        (float)db, (float)inv_dx, (float)inv_dy);
  } else {
    k_update_h<double><<<grid, block>>>(nx, ny, (double*)hz, (const double*)ex,
        (const double*)ey, (double*)psi_hz_x, (double*)psi_hz_y, (const double*)bx_h,
        (const double*)cx_h, (const double*)ikx_h, (const double*)by_h, (const double*)cy_h,
        (const double*)iky_h, db, inv_dx, inv_dy);
  }
  ++g_launches;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

int etg_update_e_te(int dtype, int nx, int ny, void* ex, void* ey, const void* hz,
                    void* psi_ex_y, void* psi_ey_x, const void* cb_ex, const void* cb_ey,
                    const void* bx_e, const void* cx_e, const void* ikx_e, const void* by_e,
                    const void* cy_e, const void* iky_e, double inv_dx, double inv_dy) {
  ETG_REQUIRE(dtype_ok(dtype) && nx > 0 && ny > 0 && nx <= 524272, ETG_ERR_ARGUMENT,  // rows of 8 on gridDim.y
              "etg_update_e_te: bad dtype %d or size %d x %d", dtype, nx, ny);
  if (fault_injected("etg_update_e_te")) return ETG_ERR_INJECTED;
  dim3 block(32, 8), grid((ny + 1 + 31) / 32, (nx + 1 + 7) / 8);
  if (dtype == ETG_F32) {
    k_update_e<float><<<grid, block>>>(nx, ny, (float*)ex, (float*)ey, (const float*)hz,
        (float*)psi_ex_y, (float*)psi_ey_x, (const float*)cb_ex, (const float*)cb_ey,
        (const float*)bx_e, (const float*)cx_e, (const float*)ikx_e, (const float*)by_e,
        (const float*)cy_e, (const float*)iky_e, (float)inv_dx, (float)inv_dy);
  } else {
    k_update_e<double><<<grid, block>>>(nx, ny, (double*)ex, (double*)ey, (const double*)hz,
        (double*)psi_ex_y, (double*)psi_ey_x, (const double*)cb_ex, (const double*)cb_ey,
        (const double*)bx_e, (const double*)cx_e, (const double*)ikx_e, (const double*)by_e,
        (const double*)cy_e, (const double*)iky_e, inv_dx, inv_dy);
  }
  ++g_launches;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

int etg_accumulate_dft(int dtype, int n_f, int n_nodes, void* acc, const void* field,
                       const int64_t* index, const void* phasors) {
  ETG_REQUIRE(dtype_ok(dtype) && n_f >= 0 && n_nodes >= 0 && n_f <= 65535, ETG_ERR_ARGUMENT,
              "etg_accumulate_dft: bad dtype %d or sizes n_f=%d n_nodes=%d", dtype, n_f, n_nodes);
  if (n_f == 0 || n_nodes == 0) return ETG_OK;
  if (fault_injected("etg_accumulate_dft")) return ETG_ERR_INJECTED;
  dim3 grid((n_nodes + 127) / 128, n_f);
  if (dtype == ETG_F32)
    k_accumulate_dft<float><<<grid, 128>>>(n_f, n_nodes, (float*)acc, (const float*)field, index,
                                           (const float*)phasors);
  else
    k_accumulate_dft<double><<<grid, 128>>>(n_f, n_nodes, (double*)acc, (const double*)field,
                                            index, (const double*)phasors);
  ++g_launches;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

int etg_scatter_sub(int dtype, int64_t n_cols, int n, void* field, const int64_t* i,
                    const int64_t* j, const void* delta) {
  ETG_REQUIRE(dtype_ok(dtype) && n >= 0 && n_cols > 0, ETG_ERR_ARGUMENT,
              "etg_scatter_sub: bad dtype %d or sizes", dtype);
  if (n == 0) return ETG_OK;
  if (fault_injected("etg_scatter_sub")) return ETG_ERR_INJECTED;
  if (dtype == ETG_F32)
    k_scatter_sub<float><<<1, 32>>>(n_cols, n, (float*)field, i, j, (const float*)delta);
  else
    k_scatter_sub<double><<<1, 32>>>(n_cols, n, (double*)field, i, j, (const double*)delta);
  ++g_launches;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

}  // extern "C"
