// One-step fused kernels of the resident simulation: the H half step (Hz + psi strips +
// magnetic sources + DFT of Hz) and the E half step (Ex, Ey + psi strips + electric
// sources + DFT of Ex, Ey), on the pitched HBM layout of etg_sim.h.
//
// Per node the arithmetic is etalon/fdtd/backends/numpy_backend.py:41-67 in its order
// (see etg_step.cu); source deltas are subtracted after the update and before the DFT,
// as etalon/fdtd/solver.py:120-128 does per step. A thread owns four consecutive nodes
// of one row (one 16-byte access per f32 array), so every node is written by one thread.
#include "etg_sim.h"

namespace etg {

// Subtract this step's delta of every source node that falls in the thread's four
// nodes (i, j0..j0+3), in the order the sources were added.
template <typename T>
__device__ __forceinline__ void apply_sources(const PhasePlan<T>& p, int comp, int i, int j0,
                                              int64_t n, T* val, int* flag) {
  for (int s = 0; s < p.n_src; ++s) {
    const SrcDesc<T>& d = p.src[s];
    if (d.comp != comp || d.i != i) continue;
    const unsigned v = (unsigned)(d.j - j0);
    if (v >= 4u) continue;
    const int64_t r = n - d.n0;
    if (r < 0 || r >= d.rows) {
      atomicOr(flag, ERRBIT_TABLE);
      continue;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (u == (int)v) val[u] = sub(val[u], d.table[r * d.stride]);
  }
}

// acc[f, k] += val * phasor[n, f] for monitor nodes among the thread's four nodes.
template <typename T>
__device__ __forceinline__ void accumulate(const PhasePlan<T>& p, int comp, int i, int j0,
                                           int64_t n, const T* val, int* flag) {
  for (int m = 0; m < p.n_mon; ++m) {
    const MonDesc<T>& d = p.mon[m];
    if (d.comp != comp) continue;
    const unsigned di = (unsigned)(i - d.ix0);
    if (di >= (unsigned)d.nxm) continue;
    if (j0 + 3 < d.jy0 || j0 >= d.jy0 + d.nym) continue;
    const int64_t r = n - d.n0;
    if (r < 0 || r >= d.rows) {
      atomicOr(flag, ERRBIT_TABLE);
      continue;
    }
    const int64_t nodes = (int64_t)d.nxm * d.nym;
    const T* ph = d.table + 2 * r * d.n_f;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const unsigned dj = (unsigned)(j0 + u - d.jy0);
      if (dj >= (unsigned)d.nym) continue;
      dft_node(d.acc, nodes, (int64_t)di * d.nym + dj, ph, d.n_f, val[u]);
    }
  }
}

// Record Hz^(n+1/2) of the thread's nodes that lie in the trace window (adjoint support).
template <typename T>
__device__ __forceinline__ void write_trace(const TraceDesc<T>& t, int i, int j0, int64_t n,
                                            const T* val, int* flag) {
  if (!t.buf) return;
  const unsigned di = (unsigned)(i - t.ti0);
  if (di >= (unsigned)t.tnx || j0 + 3 < t.tj0 || j0 >= t.tj0 + t.tny) return;
  const int64_t r = n - t.n0;
  if (r < 0 || r >= t.rows) {
    atomicOr(flag, ERRBIT_TABLE);
    return;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const unsigned dj = (unsigned)(j0 + u - t.tj0);
    if (dj < (unsigned)t.tny) t.buf[(r * t.tnx + di) * t.tny + dj] = val[u];
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_fused_h(SimArgs<T> a, PhasePlan<T> plan, int step_off) {
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int j0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (i >= a.nx || j0 >= a.ny) return;
  const int64_t row = (int64_t)i * a.P;
  Vec4<T> ex, ey0, ey1, hz;
  ex.load(a.ex + row + j0);
  const T ex4 = a.ex[row + j0 + 4];  // Ex(i, j0 + 4); inside the allocation (pitch / spare row)
  ey0.load(a.ey + row + j0);
  ey1.load(a.ey + row + a.P + j0);
  hz.load(a.hz + row + j0);
  const bool sx = i < a.xs_lo || i >= a.xs_hi;
  const T bx = a.bx_h[i], cx = a.cx_h[i], ikx = a.ikx_h[i];
#pragma unroll
  for (int v = 0; v < 4; ++v) {
    const int j = j0 + v;
    if (j >= a.ny) continue;
    const T ex_next = v < 3 ? ex.v[v + 1] : ex4;
    const T dex_dy = mul(sub(ex_next, ex.v[v]), a.inv_dy);
    const T dey_dx = mul(sub(ey1.v[v], ey0.v[v]), a.inv_dx);
    const bool sy = j < a.ys_lo || j >= a.ys_hi;
    const T psy = sy ? a.psi_hz_y[row + j] : T(0);
    const T psx = sx ? a.psi_hz_x[row + j] : T(0);
    const T py = add(mul(a.by_h[j], psy), mul(a.cy_h[j], dex_dy));
    const T px = add(mul(bx, psx), mul(cx, dey_dx));
    if (sy) a.psi_hz_y[row + j] = py;
    if (sx) a.psi_hz_x[row + j] = px;
    const T db = a.db_node ? a.db_node[row + j] : a.db;  // per node in TM mode
    hz.v[v] = add(hz.v[v], mul(db, sub(add(mul(dex_dy, a.iky_h[j]), py), add(mul(dey_dx, ikx), px))));
  }
  const int64_t n = *a.step + step_off;
  apply_sources(plan, ETG_HZ, i, j0, n, hz.v, a.flag);
  hz.store(a.hz + row + j0);
  accumulate(plan, ETG_HZ, i, j0, n, hz.v, a.flag);
  write_trace(plan.trace, i, j0, n, hz.v, a.flag);
}

template <typename T>
__global__ void __launch_bounds__(128) k_fused_e(SimArgs<T> a, PhasePlan<T> plan, int step_off) {
  const int i = blockIdx.y * blockDim.y + threadIdx.y;  // rows 0 .. nx
  const int j0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4;  // columns 0 .. ny
  if (i > a.nx || j0 > a.ny) return;
  const int64_t row = (int64_t)i * a.P;
  const bool has_ex = i < a.nx;
  const bool has_ey = i >= 1 && i < a.nx;
  Vec4<T> ex, ey, hz;
  ex.load(a.ex + row + j0);
  ey.load(a.ey + row + j0);
  hz.load(a.hz + row + j0);  // row nx of Hz is spare (zeros)
  if (has_ex) {
    Vec4<T> cb;
    cb.load(a.cb_ex + row + j0);
    T prev = j0 > 0 ? a.hz[row + j0 - 1] : T(0);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + v;
      const T here = hz.v[v];
      if (j >= 1 && j <= a.ny - 1) {
        const T d = mul(sub(here, prev), a.inv_dy);
        const bool sy = j < a.ys_lo || j >= a.ys_hi;
        const T ps = sy ? a.psi_ex_y[row + j] : T(0);
        const T p = add(mul(a.by_e[j], ps), mul(a.cy_e[j], d));
        if (sy) a.psi_ex_y[row + j] = p;
        ex.v[v] = add(ex.v[v], mul(cb.v[v], add(mul(d, a.iky_e[j]), p)));
      }
      prev = here;
    }
  }
  if (has_ey) {
    Vec4<T> cb, hzm;
    cb.load(a.cb_ey + row + j0);
    hzm.load(a.hz + row - a.P + j0);
    const bool sx = i < a.xs_lo || i >= a.xs_hi;
    const T bx = a.bx_e[i], cx = a.cx_e[i], ikx = a.ikx_e[i];
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int j = j0 + v;
      if (j >= a.ny) continue;
      const T d = mul(sub(hz.v[v], hzm.v[v]), a.inv_dx);
      const T ps = sx ? a.psi_ey_x[row + j] : T(0);
      const T p = add(mul(bx, ps), mul(cx, d));
      if (sx) a.psi_ey_x[row + j] = p;
      ey.v[v] = sub(ey.v[v], mul(cb.v[v], add(mul(d, ikx), p)));
    }
  }
  const int64_t n = *a.step + step_off;
  apply_sources(plan, ETG_EX, i, j0, n, ex.v, a.flag);
  apply_sources(plan, ETG_EY, i, j0, n, ey.v, a.flag);
  ex.store(a.ex + row + j0);
  ey.store(a.ey + row + j0);
  accumulate(plan, ETG_EX, i, j0, n, ex.v, a.flag);
  accumulate(plan, ETG_EY, i, j0, n, ey.v, a.flag);
}

template <typename T>
__global__ void k_step_add(int64_t* step, int64_t k) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += k;
}

template <typename T>
__global__ void k_check_finite(SimArgs<T> a) {
  const int64_t total = (int64_t)(a.nx + 1) * a.P;
  bool bad = false;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < total;
       k += (int64_t)gridDim.x * blockDim.x) {
    bad |= !isfinite(a.hz[k]) || !isfinite(a.ex[k]) || !isfinite(a.ey[k]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(a.flag, ERRBIT_NONFINITE);
}

template <typename T>
void launch_step_plain(const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
                       int step_off, cudaStream_t s) {
  const dim3 block(32, 4);
  const dim3 gh((a.ny + 127) / 128, (a.nx + 3) / 4);
  const dim3 ge((a.ny + 1 + 127) / 128, (a.nx + 1 + 3) / 4);
  k_fused_h<T><<<gh, block, 0, s>>>(a, ph, step_off);
  k_fused_e<T><<<ge, block, 0, s>>>(a, pe, step_off);
  g_launches += 2;
}

template <typename T>
void launch_step_add(const SimArgs<T>& a, int64_t k, cudaStream_t s) {
  k_step_add<T><<<1, 32, 0, s>>>(a.step, k);
  g_launches += 1;
}

template <typename T>
void launch_check_finite(const SimArgs<T>& a, cudaStream_t s) {
  k_check_finite<T><<<1024, 256, 0, s>>>(a);
  g_launches += 1;
}

template void launch_step_plain<float>(const SimArgs<float>&, const PhasePlan<float>&,
                                       const PhasePlan<float>&, int, cudaStream_t);
template void launch_step_plain<double>(const SimArgs<double>&, const PhasePlan<double>&,
                                        const PhasePlan<double>&, int, cudaStream_t);
template void launch_step_add<float>(const SimArgs<float>&, int64_t, cudaStream_t);
template void launch_step_add<double>(const SimArgs<double>&, int64_t, cudaStream_t);
template void launch_check_finite<float>(const SimArgs<float>&, cudaStream_t);
template void launch_check_finite<double>(const SimArgs<double>&, cudaStream_t);

}  // namespace etg
