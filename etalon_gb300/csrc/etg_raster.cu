// Permittivity staircase of boxes rasterised on the device, straight into a simulation's cb
// arrays (etalon/grid/materials.py:12-35 and etalon/fdtd/state.py:80-81): every Ex and Ey
// node takes the medium of the last box containing it (faces included, within the host's
// tolerance) or the background, and cb = Δt / (ε0 ε_r) is cast once to the run's dtype.
// Node coordinates, the containment tests and cb use the host's float64 operations in the
// host's order, so the result equals the host path bit for bit; a large design sweep then
// never builds or copies its ε maps on the host.
#include <vector>

#include "etg_sim.h"

namespace etg {

// One box: centre (cx, cy), half extents with the tolerance added (hx, hy), and ε_r.
struct RasterBox {
  double cx, cy, hx, hy, eps;
};

template <typename T>
__global__ void k_raster_cb(int n_x, int n_y, bool half_x, bool half_y, double x_min, double y_min, double dx,
                            double dy, double dt, double eps0, double background, const RasterBox* __restrict__ boxes,
                            int n_boxes, int64_t P, T* __restrict__ cb) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= n_y || i >= n_x) return;
  const double x = __dadd_rn(x_min, __dmul_rn((double)i + (half_x ? 0.5 : 0.0), dx));
  const double y = __dadd_rn(y_min, __dmul_rn((double)j + (half_y ? 0.5 : 0.0), dy));
  double eps = background;
  for (int b = 0; b < n_boxes; ++b) {
    const RasterBox q = boxes[b];
    if (fabs(__dsub_rn(x, q.cx)) <= q.hx && fabs(__dsub_rn(y, q.cy)) <= q.hy) eps = q.eps;
  }
  cb[(int64_t)i * P + j] = (T)__ddiv_rn(dt, __dmul_rn(eps0, eps));
}

}  // namespace etg

using namespace etg;

extern "C" {

int etg_sim_rasterize_cb(etg_sim* s, double x_min, double y_min, double dx, double dy, double dt, double eps0,
                         double background, int n_boxes, const double* boxes) {
  ETG_REQUIRE(s && (n_boxes == 0 || boxes) && n_boxes >= 0, ETG_ERR_ARGUMENT, "etg_sim_rasterize_cb: bad arguments");
  ETG_REQUIRE(s->nx + 1 <= 65535, ETG_ERR_ARGUMENT,
              "etg_sim_rasterize_cb: %d x rows, at most 65534 (one launch row per Ey row)", s->nx);
  ETG_REQUIRE(s->have_coeffs, ETG_ERR_STATE, "etg_sim_rasterize_cb: set the coefficients first");
  std::vector<RasterBox> host(n_boxes);
  for (int b = 0; b < n_boxes; ++b)
    host[b] = RasterBox{boxes[5 * b], boxes[5 * b + 1], boxes[5 * b + 2], boxes[5 * b + 3], boxes[5 * b + 4]};
  RasterBox* dev = nullptr;
  if (n_boxes) {
    int rc = etg_malloc((void**)&dev, n_boxes * sizeof(RasterBox));
    if (rc) return rc;
  }
  cudaError_t e = n_boxes ? cudaMemcpy(dev, host.data(), n_boxes * sizeof(RasterBox), cudaMemcpyHostToDevice)
                          : cudaSuccess;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);  // nothing still reads cb
  if (e != cudaSuccess) {
    cudaFree(dev);
    ETG_REQUIRE(false, ETG_ERR_CUDA, "etg_sim_rasterize_cb: %s", cudaGetErrorString(e));
  }
  const dim3 block(256);
  // Ex nodes: (nx, ny+1), half-cell in x; Ey nodes: (nx+1, ny), half-cell in y
  const int shapes[2][2] = {{s->nx, s->ny + 1}, {s->nx + 1, s->ny}};
  for (int c = 0; c < 2; ++c) {
    const dim3 grid((unsigned)((shapes[c][1] + 255) / 256), (unsigned)shapes[c][0]);
    if (s->dtype == ETG_F32)
      k_raster_cb<float><<<grid, block, 0, s->stream>>>(shapes[c][0], shapes[c][1], c == 0, c == 1, x_min, y_min, dx,
                                                        dy, dt, eps0, background, dev, n_boxes, s->P, (float*)s->cb[c]);
    else
      k_raster_cb<double><<<grid, block, 0, s->stream>>>(shapes[c][0], shapes[c][1], c == 0, c == 1, x_min, y_min, dx,
                                                         dy, dt, eps0, background, dev, n_boxes, s->P,
                                                         (double*)s->cb[c]);
    g_launches += 1;
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(dev);
  ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "etg_sim_rasterize_cb: %s", cudaGetErrorString(e));
  return ETG_OK;
}

int etg_sim_get_cb(etg_sim* s, int which, void* host) {
  ETG_REQUIRE(s && host && (which == 0 || which == 1), ETG_ERR_ARGUMENT, "etg_sim_get_cb: bad arguments");
  const int64_t r = which == 1 ? s->nx + 1 : s->nx, c = which == 0 ? s->ny + 1 : s->ny;
  ETG_TRY_CUDA(cudaMemcpy2DAsync(host, c * s->esize(), s->cb[which], s->P * s->esize(), c * s->esize(), r,
                                 cudaMemcpyDeviceToHost, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

}  // extern "C"
