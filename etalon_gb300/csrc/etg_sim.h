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
  T* samp;         // temporally blocked kernels: field values [step of the block][node], summed
                   // into acc after the block by k_dft_block; nullptr: accumulate in place
  int64_t n0, rows;
  int ix0, nxm, jy0, nym, n_f, comp;
};

// Trace of Hz^(n+1/2) over a window of cells, written at every H half step by the owner of
// each cell: buf[(n - n0) * tnx * tny + (i - ti0) * tny + (j - tj0)]. Used by the adjoint.
template <typename T>
struct TraceDesc {
  T* buf;  // nullptr: no trace
  int64_t n0, rows;
  int ti0, tnx, tj0, tny;
  // Recompute of an adjoint segment [n0, n0 + rows): only the trace box is wanted, so a tile
  // farther from it (in cells) than the steps left in the segment does nothing.
  int cone;
};

// Sources and monitors of one half step (H or E), passed by value as a kernel parameter.
template <typename T>
struct PhasePlan {
  int n_src, n_mon;
  SrcDesc<T> src[MAX_SRC_NODES];
  MonDesc<T> mon[MAX_MONITORS];
  TraceDesc<T> trace;  // H plan only
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
  // Per-node coefficient of the Hz-position update (pitched, nx rows of ny), replacing the
  // scalar db where set: the 2D TM mode runs its Ez update there (dt / (eps0 eps_r) per node).
  // nullptr for TE. The one-step and the temporally blocked kernels read it (not the TMA-fed).
  const T* db_node;
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

// acc[f, k] += v * ph[f] for f = 0 .. n_f-1 of one node: the adds of each accumulator keep
// their order, but the loads of eight frequencies are issued before any store, so a node's
// update costs a few memory round trips instead of one per frequency.
template <typename T>
__device__ __noinline__ void dft_node(T* __restrict__ acc, int64_t nodes, int64_t k,
                                         const T* __restrict__ ph, int n_f, T v) {
  for (int f0 = 0; f0 < n_f; f0 += 8) {
    const int m = n_f - f0 < 8 ? n_f - f0 : 8;
    T re[8], im[8], pr[8], pi[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (q < m) {
        const T* a = acc + 2 * ((f0 + q) * nodes + k);
        re[q] = a[0];
        im[q] = a[1];
        pr[q] = __ldg(ph + 2 * (f0 + q));
        pi[q] = __ldg(ph + 2 * (f0 + q) + 1);
      }
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (q < m) {
        T* a = acc + 2 * ((f0 + q) * nodes + k);
        a[0] = add(re[q], mul(v, pr[q]));
        a[1] = add(im[q], mul(v, pi[q]));
      }
  }
}

// Launchers implemented per kernel family; stream-ordered, no synchronisation.
template <typename T>
void launch_step_plain(const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
                       int step_off, cudaStream_t s);
template <typename T>
void launch_step_add(const SimArgs<T>& a, int64_t k, cudaStream_t s);
template <typename T>
void launch_check_finite(const SimArgs<T>& a, cudaStream_t s);

struct TBState;

}  // namespace etg

namespace etg {

struct Source {
  int comp;
  std::vector<int64_t> i, j;
  void* table = nullptr;  // (rows, n_nodes) dtype
  int64_t n0 = 0, rows = 0;
};

struct Monitor {
  int comp, ix0, nxm, jy0, nym, n_f;
  void* acc = nullptr;    // (n_f, nxm*nym) complex
  void* table = nullptr;  // (rows, n_f) complex
  int64_t n0 = 0, rows = 0;
  void* samp = nullptr;   // field samples of one launch block (samp_slots steps x nodes)
  int64_t samp_slots = 0;
};

// acc[f, k] += samples of steps step0 … step0 + n_slots - 1 times their phasors, in step order:
// for one thread's (frequency, node) the same additions as dft_node makes step by step. The
// table range is checked once for the block; samples and phasors of 8 steps are loaded
// before their 8 sums, so the loads overlap instead of waiting one by one.
template <typename T>
__device__ __forceinline__ void dft_block_node(const MonDesc<T>& d, int64_t q, int64_t step0, int n_slots,
                                               int* flag) {
  const int64_t nodes = (int64_t)d.nxm * d.nym;
  if (!d.samp || q >= nodes * d.n_f) return;
  const int64_t r0 = step0 - d.n0;
  if (r0 < 0 || r0 + n_slots > d.rows) {
    atomicOr(flag, ERRBIT_TABLE);
    return;
  }
  const int f = (int)(q / nodes);
  const int64_t k = q % nodes;
  T* a = d.acc + 2 * ((int64_t)f * nodes + k);
  T re = a[0], im = a[1];
  const T* smp = d.samp + k;
  const T* ph = d.table + 2 * (r0 * d.n_f + f);
  for (int s0 = 0; s0 < n_slots; s0 += 8) {
    T v[8], pr[8], pi[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (s0 + u < n_slots) {
        v[u] = smp[(int64_t)(s0 + u) * nodes];
        pr[u] = __ldg(ph + 2 * (int64_t)(s0 + u) * d.n_f);
        pi[u] = __ldg(ph + 2 * (int64_t)(s0 + u) * d.n_f + 1);
      }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (s0 + u < n_slots) {
        re = add(re, mul(v[u], pr[u]));
        im = add(im, mul(v[u], pi[u]));
      }
  }
  a[0] = re;
  a[1] = im;
}

}  // namespace etg

// The resident simulation behind the etg_sim_* entry points (internal layout).
struct etg_sim {
  using Source = etg::Source;
  using Monitor = etg::Monitor;
  using TBState = etg::TBState;
  int dtype = ETG_F32;
  int nx = 0, ny = 0;
  int64_t P = 0, rows = 0;
  void* field[7] = {};  // ETG_EX .. ETG_PSI_HZ_Y, pitched
  void* cb[2] = {};     // cb_ex, cb_ey, pitched
  void* db_node = nullptr;  // per-node Hz-position coefficient (TM mode), pitched; nullptr for TE
  void* c1d[12] = {};   // bx_e cx_e ikx_e bx_h cx_h ikx_h by_e cy_e iky_e by_h cy_h iky_h
  double db = 0, inv_dx = 0, inv_dy = 0;
  bool have_coeffs = false;
  // rows / columns whose psi may be non-zero (from c != 0, b outside (0, inf) or uploaded psi)
  std::vector<char> live_x, live_y, psi_live_x, psi_live_y;
  bool psi_dirty = false;  // stepped since the last reset: psi may be non-zero in the live rows
  std::vector<char> nonunit_x, nonunit_y;  // rows / columns whose CPML terms are not "+ 0"
  int xs_lo = 0, xs_hi = 0, ys_lo = 0, ys_hi = 0;
  int ux_lo = 0, ux_hi = 0, uy_lo = 0, uy_hi = 0;
  std::vector<Source> sources;
  std::vector<Monitor> monitors;
  int64_t* d_step = nullptr;
  int* d_flag = nullptr;
  int64_t h_step = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  int64_t last_launches = 0;
  int64_t opt[10] = {0, 0, 32, 0, 0, 0, 0, 0, 0, 0};  // 0 = default (tile shape: per dtype)
  std::map<int64_t, cudaGraphExec_t> graphs;  // keyed by steps per graph
  TBState* tb = nullptr;                      // temporally blocked kernel state
  // adjoint support: Hz trace window and whether monitors accumulate (off while recomputing)
  void* trace_buf = nullptr;
  int64_t trace_n0 = 0, trace_rows = 0;
  int trace_ti0 = 0, trace_tnx = 0, trace_tj0 = 0, trace_tny = 0;
  bool monitors_on = true;
  bool trace_cone = false;  // the trace is a segment recompute (TraceDesc::cone)
  // Output cells a batch steps: tiles whose output misses [act_i0, act_i1) x [act_j0, act_j1)
  // are left out. The adjoint narrows it to the light cone of its window while it recomputes
  // a segment; everything else runs with the whole grid.
  int act_i0 = 0, act_i1 = 1 << 30, act_j0 = 0, act_j1 = 1 << 30;

  size_t esize() const { return (size_t)dtype; }
  int64_t field_rows(int f) const { return (f == ETG_EY || f == ETG_PSI_EY_X) ? nx + 1 : nx; }
  int64_t field_cols(int f) const { return (f == ETG_EX || f == ETG_PSI_EX_Y) ? ny + 1 : ny; }
};


namespace etg {
// Internal entry points of etg_sim.cu used by the adjoint (etg_adjoint.cu).
int sim_advance_internal(etg_sim* s, int64_t n_steps);  // advance without timing or fault injection
void sim_invalidate(etg_sim* s);                        // drop graphs after a change of plans
template <typename T>
SimArgs<T> sim_args_export(etg_sim* s);                 // kernel arguments of the simulation
template <typename T>
int sim_plans_export(etg_sim* s, PhasePlan<T>* ph, PhasePlan<T>* pe,  // its source/monitor plans;
                     int64_t sample_slots = 0);                        // > 0: monitors sample per block
int64_t sim_sample_slots(const etg_sim* s);             // block length the sample buffers must hold
int sim_check_tables(etg_sim* s, int64_t n_steps);      // tables cover the next n_steps steps
}  // namespace etg
