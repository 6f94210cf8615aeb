// etg_tb_advance_static: the temporally blocked advance for callers that cannot allocate
// device memory.
//
// Some callers of this library cannot call cudaMalloc when they step fields: an embedding
// application that owns all device memory through its own fixed arena and allows no other
// allocations, a process that runs under a hard device-memory budget where a late allocation
// could fail mid-run, or a latency-sensitive loop that cannot afford the device-wide
// synchronisation that cudaMalloc and cudaFree imply. This entry point steps fields the caller
// already owns and keeps everything else it needs — the second buffer of the ping-pong pair,
// the tile list and the step counter — in one file-scope __device__ array of
// ETG_STATIC_SCRATCH_BYTES. Every GPU that loads the library holds that array until the
// process exits.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "etg_tb.h"

namespace etg {
namespace {

// Scratch of etg_tb_advance_static: [7 field/psi planes][int64 step][int flag][pad][tiles].
// Shared by every call; it keeps the last call's contents.
static __device__ __align__(256) unsigned char g_static_scratch[ETG_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device, looked up once per device.
// In host code the array's name is only a host-side stand-in, so kernels get this address.
int scratch_address(void** out) {
  int dev = 0;
  ETG_TRY_CUDA(cudaGetDevice(&dev));
  ETG_REQUIRE(dev >= 0 && dev < kMaxDevices, ETG_ERR_ARGUMENT, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    ETG_REQUIRE(e == cudaSuccess && p, ETG_ERR_CUDA,
                "cudaGetSymbolAddress of the static scratch failed on device %d: %s", dev,
                cudaGetErrorString(e));
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return ETG_OK;
}

// Longest run of indices not marked: [lo, hi).
void longest_run(const std::vector<char>& marked, int* lo, int* hi) {
  const int n = (int)marked.size();
  int best_lo = 0, best_len = -1, run_lo = 0;
  for (int k = 0; k <= n; ++k)
    if (k == n || marked[k]) {
      if (k - run_lo > best_len) {
        best_len = k - run_lo;
        best_lo = run_lo;
      }
      run_lo = k + 1;
    }
  *lo = best_lo;
  *hi = best_lo + std::max(best_len, 0);
}

template <typename T>
int host_copy(std::vector<T>* out, const void* dev, int64_t n) {
  out->resize(n);
  ETG_TRY_CUDA(cudaMemcpy(out->data(), dev, n * sizeof(T), cudaMemcpyDeviceToHost));
  return ETG_OK;
}

template <typename T>
int advance_static(int nx, int ny, int64_t pitch, void* const f[7], const void* cb_ex,
                   const void* cb_ey, const void* const c[12], double db, double inv_dx,
                   double inv_dy, int64_t n_steps) {
  // size check first, before any device access: the tile count of the default shape bounds
  // the tile list whatever the interior/CPML split (one column more for a shifted first column)
  int ER, EC, K;
  tb_default_shape((int)sizeof(T), &ER, &EC, &K);
  const int64_t tiles_max = (int64_t)((nx + 1 + ER - 2 * K - 1) / (ER - 2 * K)) *
                            ((ny + 1 + EC - 2 * K - 1) / (EC - 2 * K) + 1);
  const size_t plane = (size_t)(nx + 2) * pitch * sizeof(T);
  const size_t counters = 7 * plane, tiles_at = counters + 256;
  const size_t need = tiles_at + (size_t)tiles_max * sizeof(int2);
  ETG_REQUIRE(need <= ETG_STATIC_SCRATCH_BYTES, ETG_ERR_ARGUMENT,
              "etg_tb_advance_static: a %d x %d grid (pitch %lld) needs %zu bytes of scratch, more "
              "than the %d bytes this entry point holds; use etg_sim_* for larger grids",
              nx, ny, (long long)pitch, need, (int)ETG_STATIC_SCRATCH_BYTES);

  // CPML strips and the unit rectangle from the 1D profiles (psi is +0 where c = 0).
  std::vector<T> h[12];
  const int64_t len[12] = {nx + 1, nx + 1, nx + 1, nx, nx, nx, ny + 1, ny + 1, ny + 1, ny, ny, ny};
  for (int k = 0; k < 12; ++k) {
    int rc = host_copy(&h[k], c[k], len[k]);
    if (rc) return rc;
  }
  auto live = [](T b, T cc) { return !(cc == T(0)) || !(b > T(0)) || !std::isfinite((double)b); };
  std::vector<char> lx(nx + 1, 0), ly(ny + 1, 0), ux(nx + 1, 0), uy(ny + 1, 0);
  for (int i = 0; i < nx; ++i) {
    lx[i] |= live(h[3][i], h[4][i]);
    ux[i] |= !(h[5][i] == T(1));
  }
  for (int i = 1; i < nx; ++i) {
    lx[i] |= live(h[0][i], h[1][i]);
    ux[i] |= !(h[2][i] == T(1));
  }
  for (int j = 0; j < ny; ++j) {
    ly[j] |= live(h[9][j], h[10][j]);
    uy[j] |= !(h[11][j] == T(1));
  }
  for (int j = 1; j < ny; ++j) {
    ly[j] |= live(h[6][j], h[7][j]);
    uy[j] |= !(h[8][j] == T(1));
  }
  SimArgs<T> a;
  memset(&a, 0, sizeof a);
  a.nx = nx;
  a.ny = ny;
  a.P = pitch;
  longest_run(lx, &a.xs_lo, &a.xs_hi);
  longest_run(ly, &a.ys_lo, &a.ys_hi);
  for (int k = 0; k <= nx; ++k) ux[k] |= lx[k];
  for (int k = 0; k <= ny; ++k) uy[k] |= ly[k];
  longest_run(ux, &a.ux_lo, &a.ux_hi);
  longest_run(uy, &a.uy_lo, &a.uy_hi);

  std::vector<int2> tiles;
  int n_inner = 0;
  tb_tiles((int)sizeof(T), nx, ny, a.ux_lo, a.ux_hi, a.uy_lo, a.uy_hi, &tiles, &n_inner);
  const int n_pml = (int)tiles.size() - n_inner;
  ETG_REQUIRE((int64_t)tiles.size() <= tiles_max, ETG_ERR_STATE, "tile count above its bound");

  unsigned char* base = nullptr;
  int rc = scratch_address((void**)&base);
  if (rc) return rc;
  const cudaStream_t s = 0;  // the default stream: calls return when their work is done
  // The seven planes of the second buffer, the step counter and the error flag start at zero,
  // as the allocating engine's second buffer does: corner tiles read psi over their whole
  // extended tile, so halo cells that no launch writes must not keep an earlier call's bytes
  // (another grid, pitch or precision).
  ETG_TRY_CUDA(cudaMemsetAsync(base, 0, counters + 256, s));
  ETG_TRY_CUDA(cudaMemcpyAsync(base + tiles_at, tiles.data(), tiles.size() * sizeof(int2),
                               cudaMemcpyHostToDevice, s));

  a.ex = (T*)f[ETG_EX];
  a.ey = (T*)f[ETG_EY];
  a.hz = (T*)f[ETG_HZ];
  a.psi_ex_y = (T*)f[ETG_PSI_EX_Y];
  a.psi_ey_x = (T*)f[ETG_PSI_EY_X];
  a.psi_hz_x = (T*)f[ETG_PSI_HZ_X];
  a.psi_hz_y = (T*)f[ETG_PSI_HZ_Y];
  a.cb_ex = (const T*)cb_ex;
  a.cb_ey = (const T*)cb_ey;
  const T** cp[12] = {&a.bx_e, &a.cx_e, &a.ikx_e, &a.bx_h, &a.cx_h, &a.ikx_h,
                      &a.by_e, &a.cy_e, &a.iky_e, &a.by_h, &a.cy_h, &a.iky_h};
  for (int k = 0; k < 12; ++k) *cp[k] = (const T*)c[k];
  a.db = (T)db;
  a.inv_dx = (T)inv_dx;
  a.inv_dy = (T)inv_dy;
  a.step = (int64_t*)(base + counters);
  a.flag = (int*)(base + counters + sizeof(int64_t));
  SimArgs<T> b = a;  // the second buffer: seven planes of the scratch
  T** bp[7] = {&b.ex, &b.ey, &b.hz, &b.psi_ex_y, &b.psi_ey_x, &b.psi_hz_x, &b.psi_hz_y};
  for (int k = 0; k < 7; ++k) *bp[k] = (T*)(base + k * plane);
  const int2* d_tiles = (const int2*)(base + tiles_at);

  // Launch offsets are relative to the device step counter and fit an int: the counter is
  // advanced every kPairsPerAdd pairs, so any 64-bit step count is covered.
  constexpr int64_t kPairsPerAdd = 1 << 20;
  const int64_t pairs = n_steps / (2 * K);
  for (int64_t p0 = 0; p0 < pairs; p0 += kPairsPerAdd) {
    const int64_t np = std::min(kPairsPerAdd, pairs - p0);
    for (int64_t p = 0; p < np; ++p) {
      ETG_TRY_CUDA(tb_default_launch<T>(a, b, d_tiles, n_inner, n_pml, (int)(2 * K * p), s));
      ETG_TRY_CUDA(tb_default_launch<T>(b, a, d_tiles, n_inner, n_pml, (int)(2 * K * p + K), s));
    }
    launch_step_add<T>(a, 2 * K * np, s);
  }
  PhasePlan<T> none;
  memset(&none, 0, sizeof none);
  const int64_t rem = n_steps - 2 * K * pairs;
  for (int64_t k = 0; k < rem; ++k) launch_step_plain<T>(a, none, none, (int)k, s);
  if (rem) launch_step_add<T>(a, rem, s);
  ETG_LAUNCH_CHECK();
  ETG_TRY_CUDA(cudaStreamSynchronize(s));
  int flag = 0;
  ETG_TRY_CUDA(cudaMemcpy(&flag, a.flag, sizeof flag, cudaMemcpyDeviceToHost));
  ETG_REQUIRE(flag == 0, ETG_ERR_STATE, "etg_tb_advance_static: device error flags 0x%x", flag);
  return ETG_OK;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace
}  // namespace etg

using namespace etg;

extern "C" int etg_tb_advance_static(int dtype, int nx, int ny, int64_t pitch, void* ex, void* ey,
                                     void* hz, void* psi_ex_y, void* psi_ey_x, void* psi_hz_x,
                                     void* psi_hz_y, const void* cb_ex, const void* cb_ey,
                                     const void* bx_e, const void* cx_e, const void* ikx_e,
                                     const void* bx_h, const void* cx_h, const void* ikx_h,
                                     const void* by_e, const void* cy_e, const void* iky_e,
                                     const void* by_h, const void* cy_h, const void* iky_h,
                                     double db, double inv_dx, double inv_dy, int64_t n_steps) {
  ETG_REQUIRE(dtype_ok(dtype), ETG_ERR_ARGUMENT, "etg_tb_advance_static: dtype must be 4 or 8, got %d", dtype);
  ETG_REQUIRE(nx >= 2 && ny >= 2 && nx < (1 << 20) && ny < (1 << 20) && n_steps >= 0, ETG_ERR_ARGUMENT,
              "etg_tb_advance_static: grid %d x %d or step count %lld out of range", nx, ny, (long long)n_steps);
  ETG_REQUIRE(pitch >= (int64_t)ny + 1 && pitch % 32 == 0, ETG_ERR_ARGUMENT,
              "etg_tb_advance_static: pitch %lld must be a multiple of 32 and at least ny + 1 = %d",
              (long long)pitch, ny + 1);
  void* const f[7] = {ex, ey, hz, psi_ex_y, psi_ey_x, psi_hz_x, psi_hz_y};
  const void* const c[12] = {bx_e, cx_e, ikx_e, bx_h, cx_h, ikx_h, by_e, cy_e, iky_e, by_h, cy_h, iky_h};
  for (void* p : f)
    ETG_REQUIRE(p && aligned16(p), ETG_ERR_ARGUMENT, "etg_tb_advance_static: field pointers must be 16-byte aligned device pointers");
  ETG_REQUIRE(cb_ex && cb_ey && aligned16(cb_ex) && aligned16(cb_ey), ETG_ERR_ARGUMENT,
              "etg_tb_advance_static: cb pointers must be 16-byte aligned device pointers");
  for (const void* p : c) ETG_REQUIRE(p, ETG_ERR_ARGUMENT, "etg_tb_advance_static: null coefficient array");
  if (n_steps == 0) return ETG_OK;
  return dtype == ETG_F32 ? advance_static<float>(nx, ny, pitch, f, cb_ex, cb_ey, c, db, inv_dx, inv_dy, n_steps)
                          : advance_static<double>(nx, ny, pitch, f, cb_ex, cb_ey, c, db, inv_dx, inv_dy, n_steps);
}
