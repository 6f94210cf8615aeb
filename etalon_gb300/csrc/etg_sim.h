// Internal layout of a resident simulation (etg_sim) shared by its kernels.
#pragma once

#include <map>
#include <vector>

#include "etg_common.cuh"

namespace etg {

constexpr int MAX_SRC_NODES = 32;  // point-source nodes per phase (bilinear: 4 per source)
constexpr int MAX_MONITORS = 24;   // monitor components per phase

// One source node: the value subtracted at step n is table[(n - n0) * stride].
template <typename T>
struct SrcDesc {
  const T* table;
  int64_t n0, rows;
  int i, j, stride, comp;
};

// One monitor component: a node rectangle, its accumulator and phasor rows.
template <typename T>
struct MonDesc {
  T* acc;          // (n_f, nxm*nym) complex
  const T* table;  // (rows, n_f) complex
  int64_t n0, rows;
  int ix0, nxm, jy0, nym, n_f, comp;
};

// Sources and monitors of one half step (H or E), passed by value as a kernel parameter.
template <typename T>
struct PhasePlan {
  int n_src, n_mon;
  SrcDesc<T> src[MAX_SRC_NODES];
  MonDesc<T> mon[MAX_MONITORS];
};

// Fields and coefficients in HBM. Every 2D array has rows of pitch P elements (P a
// multiple of 32, >= ny + 1) and nx + 2 rows; Hz/Ex/Ey/psi share the index i * P + j.
template <typename T>
struct SimArgs {
  int nx, ny;
  int64_t P;
  T *ex, *ey, *hz, *psi_ex_y, *psi_ey_x, *psi_hz_x, *psi_hz_y;
  const T *cb_ex, *cb_ey;
  const T *bx_e, *cx_e, *ikx_e, *bx_h, *cx_h, *ikx_h, *by_e, *cy_e, *iky_e, *by_h, *cy_h, *iky_h;
  T db, inv_dx, inv_dy;
  // CPML strips: rows i < xs_lo or i >= xs_hi, columns j < ys_lo or j >= ys_hi carry psi;
  // everywhere else psi is exactly +0 and is neither read nor written.
  int xs_lo, xs_hi, ys_lo, ys_hi;
  // Unit rectangle: rows [ux_lo, ux_hi) x columns [uy_lo, uy_hi) have c = 0, b > 0 and
  // 1/kappa = 1 exactly and no psi, so the CPML terms of their update reduce to "+ 0".
  int ux_lo, ux_hi, uy_lo, uy_hi;
  int64_t* step;  // device step counter n of the first step of a launch block
  int* flag;      // device error bits (ERRBIT_*)
};

constexpr int ERRBIT_TABLE = 1;      // a source or phasor table did not cover a step
constexpr int ERRBIT_NONFINITE = 2;  // NaN/Inf seen by the finiteness check
constexpr int ERRBIT_TIMEOUT = 4;    // a bounded wait gave up

// Launchers implemented per kernel family; stream-ordered, no synchronisation.
template <typename T>
void launch_step_plain(const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
                       int step_off, cudaStream_t s);
template <typename T>
void launch_step_add(const SimArgs<T>& a, int64_t k, cudaStream_t s);
template <typename T>
void launch_check_finite(const SimArgs<T>& a, cudaStream_t s);

}  // namespace etg
