// Discrete adjoint of the 2D TE leapfrog (no counterpart in Etalon): dJ/dcb over a design
// window, for an objective J of the DFT monitor accumulators.
//
// Forward step n (etalon/fdtd/solver.py:120-128, numpy_backend.py:41-67):
//   H:  A_y = dEx/dy·iky_h + psi_hz_y',  A_x = dEy/dx·ikx_h + psi_hz_x',  Hz' = Hz + db (A_y - A_x)
//   E:  Ex' = Ex + cb_ex (dHz/dy·iky_e + psi_ex_y'),  Ey' = Ey - cb_ey (dHz/dx·ikx_e + psi_ey_x')
//   with psi' = b psi + c d and d the scaled differences; then sources and DFTs.
// The reverse sweep runs n = N-1 … 0 with lambda = dJ/d(state) and two kernels per step:
//   RE(n): lambda_Hz(n+1/2) += transpose(E update) + DFT-H source, lambda_psi_e updated,
//          dJ/dcb += lambda_E(n+1) · C^n on the design window, C^n from the recorded Hz trace;
//   RH(n): lambda_E(n) += transpose(H update) + DFT-E source of step n-1, lambda_psi_h updated.
// The adjoint of a DFT term acc += v·ph is dJ/dv = Re(G)·Re(ph) + Im(G)·Im(ph), G = dJ/dacc.
// Every scaled difference of the forward appears once in each transposed gather, so each
// thread recomputes the neighbour's term; lambda_psi is double-buffered for that.
//
// What the gradient needs from the forward is Hz^(n+1/2) on the design window plus one cell
// of halo at every step. The forward either records it for all steps ("trace" mode) or keeps
// full-state checkpoints every S ~ sqrt(N) steps and re-records it segment by segment in the
// reverse sweep ("checkpoint" mode); both give the same bits.
#include <algorithm>
#include <map>
#include <cmath>
#include <cstring>
#include <vector>

#include "etg_sim.h"
#include "etg_tb.h"
#include "etg_tb_adj.h"

namespace etg {

// One DFT monitor with its objective gradient G = dJ/dacc (n_f, nodes) complex.
template <typename T>
struct AdjMon {
  const T* table;  // phasor rows (rows, n_f) complex
  const T* g;      // (n_f, nxm*nym) complex
  int64_t n0, rows;
  int ix0, nxm, jy0, nym, n_f, comp;
};

template <typename T>
struct AdjPlan {
  int n_mon;
  AdjMon<T> mon[MAX_MONITORS];
};

template <typename T>
struct AdjArgs {
  SimArgs<T> s;                      // geometry, coefficients, strips of the simulation
  T *lex, *ley, *lhz;                // adjoint fields, pitched like the fields
  const T *lpsi_in[4];               // psi_hz_x, psi_hz_y, psi_ex_y, psi_ey_x (this sweep's input)
  T* lpsi_out[4];
  const T* trace;                    // Hz^(n+1/2) on [ti0, ti0+tnx) x [tj0, tj0+tny) per step
  int64_t trace_n0;
  int ti0, tnx, tj0, tny;
  int i0, nxd, j0, nyd;              // design cells
  double *gx, *gy;                   // dJ/dcb_ex (nxd, nyd+1), dJ/dcb_ey (nxd+1, nyd)
};

// Sum_f Re(G)·Re(ph) + Im(G)·Im(ph) for node (i, j) of component comp, if monitored.
template <typename T>
__device__ __forceinline__ T adj_source(const AdjPlan<T>& p, int comp, int i, int j, int64_t n) {
  T acc = T(0);
  for (int m = 0; m < p.n_mon; ++m) {
    const AdjMon<T>& d = p.mon[m];
    if (d.comp != comp) continue;
    const unsigned di = (unsigned)(i - d.ix0), dj = (unsigned)(j - d.jy0);
    if (di >= (unsigned)d.nxm || dj >= (unsigned)d.nym) continue;
    const int64_t r = n - d.n0;
    if (r < 0 || r >= d.rows) continue;  // the host checks table coverage before the sweep
    const int64_t nodes = (int64_t)d.nxm * d.nym, k = (int64_t)di * d.nym + dj;
    const T* ph = d.table + 2 * r * d.n_f;
    for (int f = 0; f < d.n_f; ++f) {
      const T* g = d.g + 2 * (f * nodes + k);
      acc = acc + g[0] * ph[2 * f] + g[1] * ph[2 * f + 1];
    }
  }
  return acc;
}

// Transposed E update of the Ex node (i, j): returns dJ/d(dHz/dy) and updates lambda_psi_ex_y.
template <typename T>
__device__ __forceinline__ T gx_at(const AdjArgs<T>& a, int i, int j, bool own) {
  const SimArgs<T>& s = a.s;
  if (j < 1 || j > s.ny - 1 || i < 0 || i >= s.nx) return T(0);
  const int64_t g = (int64_t)i * s.P + j;
  const T lc = s.cb_ex[g] * a.lex[g];
  if (j < s.ys_lo || j >= s.ys_hi) {
    const T lpt = a.lpsi_in[2][g] + lc;
    if (own) a.lpsi_out[2][g] = s.by_e[j] * lpt;
    return s.iky_e[j] * lc + s.cy_e[j] * lpt;
  }
  return s.iky_e[j] * lc;
}

// Transposed E update of the Ey node (i, j): returns dJ/d(dHz/dx) and updates lambda_psi_ey_x.
template <typename T>
__device__ __forceinline__ T gy_at(const AdjArgs<T>& a, int i, int j, bool own) {
  const SimArgs<T>& s = a.s;
  if (i < 1 || i > s.nx - 1 || j < 0 || j >= s.ny) return T(0);
  const int64_t g = (int64_t)i * s.P + j;
  const T lc = -(s.cb_ey[g] * a.ley[g]);
  if (i < s.xs_lo || i >= s.xs_hi) {
    const T lpt = a.lpsi_in[3][g] + lc;
    if (own) a.lpsi_out[3][g] = s.bx_e[i] * lpt;
    return s.ikx_e[i] * lc + s.cx_e[i] * lpt;
  }
  return s.ikx_e[i] * lc;
}

template <typename T>
__global__ void __launch_bounds__(128) k_adj_re(AdjArgs<T> a, AdjPlan<T> ph, int64_t n) {
  const SimArgs<T>& s = a.s;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.nx || j >= s.ny) return;
  const int64_t g = (int64_t)i * s.P + j;
  const T gx0 = gx_at(a, i, j, true), gx1 = gx_at(a, i, j + 1, false);
  const T gy0 = gy_at(a, i, j, true), gy1 = gy_at(a, i + 1, j, false);
  a.lhz[g] = a.lhz[g] + s.inv_dy * (gx0 - gx1) + s.inv_dx * (gy0 - gy1) + adj_source(ph, ETG_HZ, i, j, n);
  // dJ/dcb on the design window: Ex' = Ex + cb·C, Ey' = Ey - cb·C, C as the forward rounds it
  const int64_t r = n - a.trace_n0;
  const int ri = i - a.ti0, rj = j - a.tj0;
  const T* tr = a.trace + r * a.tnx * a.tny;
  if (i >= a.i0 && i < a.i0 + a.nxd && j >= a.j0 && j <= a.j0 + a.nyd) {
    const T c = add(mul(sub(tr[ri * a.tny + rj], tr[ri * a.tny + rj - 1]), s.inv_dy), T(0));
    a.gx[(int64_t)(i - a.i0) * (a.nyd + 1) + (j - a.j0)] += (double)a.lex[g] * (double)c;
  }
  if (i >= a.i0 && i <= a.i0 + a.nxd && j >= a.j0 && j < a.j0 + a.nyd) {
    const T c = add(mul(sub(tr[ri * a.tny + rj], tr[(ri - 1) * a.tny + rj]), s.inv_dx), T(0));
    a.gy[(int64_t)(i - a.i0) * a.nyd + (j - a.j0)] -= (double)a.ley[g] * (double)c;
  }
}

// Transposed H update of the Hz cell (i, j): dJ/d(dEx/dy), dJ/d(dEy/dx); updates lambda_psi_h.
template <typename T>
__device__ __forceinline__ void h_at(const AdjArgs<T>& a, int i, int j, bool own, T* hx, T* hy) {
  const SimArgs<T>& s = a.s;
  if (i < 0 || i >= s.nx || j < 0 || j >= s.ny) {
    *hx = *hy = T(0);
    return;
  }
  const int64_t g = (int64_t)i * s.P + j;
  const T la = s.db * a.lhz[g];
  if (j < s.ys_lo || j >= s.ys_hi) {
    const T lpt = a.lpsi_in[1][g] + la;
    if (own) a.lpsi_out[1][g] = s.by_h[j] * lpt;
    *hx = s.iky_h[j] * la + s.cy_h[j] * lpt;
  } else {
    *hx = s.iky_h[j] * la;
  }
  if (i < s.xs_lo || i >= s.xs_hi) {
    const T lpt = a.lpsi_in[0][g] - la;
    if (own) a.lpsi_out[0][g] = s.bx_h[i] * lpt;
    *hy = -(s.ikx_h[i] * la) + s.cx_h[i] * lpt;
  } else {
    *hy = -(s.ikx_h[i] * la);
  }
}

template <typename T>
__global__ void __launch_bounds__(128) k_adj_rh(AdjArgs<T> a, AdjPlan<T> pe, int64_t n_src) {
  const SimArgs<T>& s = a.s;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;  // rows 0 .. nx
  const int j = blockIdx.x * blockDim.x + threadIdx.x;  // columns 0 .. ny
  if (i > s.nx || j > s.ny) return;
  const int64_t g = (int64_t)i * s.P + j;
  T hx0, hy0, hxl, hyl, hxu, hyu;
  h_at(a, i, j, true, &hx0, &hy0);
  h_at(a, i, j - 1, false, &hxl, &hyl);
  h_at(a, i - 1, j, false, &hxu, &hyu);
  if (i < s.nx) {  // Ex(i, j), j in [0, ny]
    T v = a.lex[g] + s.inv_dy * (hxl - hx0);
    if (n_src >= 0) v = v + adj_source(pe, ETG_EX, i, j, n_src);
    a.lex[g] = v;
  }
  if (j < s.ny) {  // Ey(i, j), i in [0, nx]
    T v = a.ley[g] + s.inv_dx * (hyu - hy0);
    if (n_src >= 0) v = v + adj_source(pe, ETG_EY, i, j, n_src);
    a.ley[g] = v;
  }
}

// lambda_E += DFT-E source of step n (the last step, before the sweep starts).
template <typename T>
__global__ void k_adj_esrc(AdjArgs<T> a, AdjPlan<T> pe, int64_t n) {
  const SimArgs<T>& s = a.s;
  const int i = blockIdx.y * blockDim.y + threadIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (i > s.nx || j > s.ny) return;
  const int64_t g = (int64_t)i * s.P + j;
  if (i < s.nx) a.lex[g] = a.lex[g] + adj_source(pe, ETG_EX, i, j, n);
  if (j < s.ny) a.ley[g] = a.ley[g] + adj_source(pe, ETG_EY, i, j, n);
}

// One rectangle of one plane, in 32-bit words: dst[r * dst_pitch + w] = src[r * src_pitch + w]
// for r < rows, w < words, with src and dst advanced by src_k and dst_k words per checkpoint
// index k. `step`, when set, receives the launch's step value (a restored simulation).
struct RectCopy {
  const uint32_t* src;
  uint32_t* dst;
  int64_t src_pitch, dst_pitch, src_k, dst_k;
  int64_t* step;
  int rows, words;
};

__global__ void k_copy_rects(const RectCopy* __restrict__ copies, int64_t k, int64_t step_value) {
  const RectCopy c = copies[blockIdx.y];
  const uint32_t* src = c.src + k * c.src_k;
  uint32_t* dst = c.dst + k * c.dst_k;
  const int64_t n = (int64_t)c.rows * c.words;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = q / c.words, w = q % c.words;
    dst[r * c.dst_pitch + w] = src[r * c.src_pitch + w];
  }
  if (c.step && blockIdx.x == 0 && threadIdx.x == 0) *c.step = step_value;
}

// Per-node tables of the adjoint sources: tables[q * n_steps + n] = adj_source(plan, node q, n),
// the exact sum the one-step kernels add at that node and step.
template <typename T>
__global__ void k_adj_tables(AdjPlan<T> plan, const int4* __restrict__ nodes, int n_nodes, int64_t n_steps,
                             T* __restrict__ tables) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= (int64_t)n_nodes * n_steps) return;
  const int q = (int)(k / n_steps);
  const int64_t n = k % n_steps;
  const int4 d = nodes[q];  // i, j, comp
  tables[k] = adj_source(plan, d.z, d.x, d.y, n);
}

}  // namespace etg

using namespace etg;

// Launch pairs per captured block of the batched reverse sweep.
constexpr int64_t kBatchPairsPerGraph = 4;

struct etg_adj {
  etg_sim* sim = nullptr;
  int i0 = 0, nxd = 0, j0 = 0, nyd = 0;
  int ti0 = 0, tnx = 0, tj0 = 0, tny = 0;
  int64_t n_steps = 0, stride = 0;  // stride 0: trace of every step
  void* trace = nullptr;
  size_t trace_cap = 0;
  // checkpoints: nseg x 7 planes of the light-cone rectangle [ck_r0, ck_r1) x [ck_c0, ck_c1)
  // (elements of the pitched planes), stored compactly one after the other
  void* ckpt = nullptr;
  size_t ckpt_cap = 0;
  int64_t ck_r0 = 0, ck_r1 = 0, ck_c0 = 0, ck_c1 = 0;
  void* d_copies = nullptr;  // the RectCopy list of the current save or restore
  size_t copies_cap = 0;
  void* lam[3] = {};        // lambda Ex, Ey, Hz
  void* lpsi[2][4] = {};    // double-buffered lambda psi
  double* grad = nullptr;   // gx then gy
  std::vector<void*> gacc;  // per monitor, device G
  // temporally blocked sweep: second lambda buffer, tiles, adjoint-source tables
  void* alt[7] = {};
  int2* tiles = nullptr;
  std::vector<int2> h_tiles;
  int n_inner = 0, n_pml = 0;
  void* tables = nullptr;
  size_t tables_bytes = 0;
  std::vector<int4> hnodes, enodes;  // i, j, comp
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaStream_t sides[3] = {};                    // one branch per CPML kind
  cudaEvent_t joins[3] = {};
  int n_kind[3] = {};                            // CPML tiles of each kind (the list is sorted by kind)
  int64_t* d_ctl = nullptr;                      // top step of the launch block, trace origin
  std::map<int64_t, cudaGraphExec_t> graphs;     // key: pairs per graph * 2 + lambda-psi parity
  etg_batch* fwd1 = nullptr;                     // segment recompute with the plans in device memory
  void* ltrace = nullptr;                        // lambda E of the window per step of a launch block
  int64_t ltrace_slots = 0;
  void* d_args1 = nullptr;                       // device copy of the block's TBAdjArgs (gradient kernel)
};

namespace {

size_t plane_bytes(const etg_sim* s) { return (size_t)s->rows * s->P * s->esize(); }

int ensure(void** p, size_t bytes) {
  if (*p) return ETG_OK;
  return etg_malloc(p, bytes);
}

template <typename T>
AdjArgs<T> adj_args(etg_adj* A, SimArgs<T> sa, int par_e, int par_h, int64_t trace_n0) {
  AdjArgs<T> a;
  memset(&a, 0, sizeof a);
  a.s = sa;
  a.lex = (T*)A->lam[0];
  a.ley = (T*)A->lam[1];
  a.lhz = (T*)A->lam[2];
  for (int k = 0; k < 4; ++k) {
    const int par = k < 2 ? par_h : par_e;
    a.lpsi_in[k] = (const T*)A->lpsi[par][k];
    a.lpsi_out[k] = (T*)A->lpsi[1 - par][k];
  }
  a.trace = (const T*)A->trace;
  a.trace_n0 = trace_n0;
  a.ti0 = A->ti0;
  a.tnx = A->tnx;
  a.tj0 = A->tj0;
  a.tny = A->tny;
  a.i0 = A->i0;
  a.nxd = A->nxd;
  a.j0 = A->j0;
  a.nyd = A->nyd;
  a.gx = A->grad;
  a.gy = A->grad + (size_t)A->nxd * (A->nyd + 1);
  return a;
}

template <typename T>
SimArgs<T> sim_args_of(etg_sim* s) {
  SimArgs<T> a;
  memset(&a, 0, sizeof a);
  a.nx = s->nx;
  a.ny = s->ny;
  a.P = s->P;
  a.ex = (T*)s->field[ETG_EX];
  a.ey = (T*)s->field[ETG_EY];
  a.hz = (T*)s->field[ETG_HZ];
  a.cb_ex = (const T*)s->cb[0];
  a.cb_ey = (const T*)s->cb[1];
  const T** c[12] = {&a.bx_e, &a.cx_e, &a.ikx_e, &a.bx_h, &a.cx_h, &a.ikx_h,
                     &a.by_e, &a.cy_e, &a.iky_e, &a.by_h, &a.cy_h, &a.iky_h};
  for (int k = 0; k < 12; ++k) *c[k] = (const T*)s->c1d[k];
  a.db = (T)s->db;
  a.inv_dx = (T)s->inv_dx;
  a.inv_dy = (T)s->inv_dy;
  a.xs_lo = s->xs_lo;
  a.xs_hi = s->xs_hi;
  a.ys_lo = s->ys_lo;
  a.ys_hi = s->ys_hi;
  a.step = s->d_step;
  a.flag = s->d_flag;
  return a;
}

void set_trace(etg_sim* s, void* buf, int64_t n0, int64_t rows, const etg_adj* A) {
  s->trace_buf = buf;
  s->trace_n0 = n0;
  s->trace_rows = rows;
  s->trace_ti0 = A->ti0;
  s->trace_tnx = A->tnx;
  s->trace_tj0 = A->tj0;
  s->trace_tny = A->tny;
  sim_invalidate(s);
}

void clear_trace(etg_sim* s) {
  s->trace_buf = nullptr;
  s->trace_cone = false;
  sim_invalidate(s);
}

// Arguments of one temporally blocked launch; `to_alt` reads the primary lambda buffers
// (lambda psi of the current parities) and writes the second buffer, else the reverse.
template <typename T>
TBAdjArgs<T> tb_adj_args(etg_adj* A, const SimArgs<T>& sa, int par_e, int par_h, const int64_t* ctl, bool to_alt) {
  TBAdjArgs<T> a;
  memset(&a, 0, sizeof a);
  a.s = sa;
  void* prim[7] = {A->lam[0], A->lam[1], A->lam[2], A->lpsi[par_h][0], A->lpsi[par_h][1], A->lpsi[par_e][2],
                   A->lpsi[par_e][3]};
  for (int k = 0; k < 7; ++k) {
    a.in[k] = (const T*)(to_alt ? prim[k] : A->alt[k]);
    a.out[k] = (T*)(to_alt ? A->alt[k] : prim[k]);
  }
  a.trace = (const T*)A->trace;
  a.ctl = ctl;
  a.ti0 = A->ti0;
  a.tnx = A->tnx;
  a.tj0 = A->tj0;
  a.tny = A->tny;
  a.i0 = A->i0;
  a.nxd = A->nxd;
  a.j0 = A->j0;
  a.nyd = A->nyd;
  a.gx = A->grad;
  a.gy = A->grad + (size_t)A->nxd * (A->nyd + 1);
  a.ltrace = (T*)A->ltrace;
  const int64_t N = A->n_steps;
  a.n_hsrc = (int)A->hnodes.size();
  a.n_esrc = (int)A->enodes.size();
  for (int q = 0; q < a.n_hsrc; ++q)
    a.hsrc[q] = AdjSrc<T>{(const T*)A->tables + q * N, A->hnodes[q].x, A->hnodes[q].y, A->hnodes[q].z};
  for (int q = 0; q < a.n_esrc; ++q)
    a.esrc[q] = AdjSrc<T>{(const T*)A->tables + (a.n_hsrc + q) * N, A->enodes[q].x, A->enodes[q].y,
                          A->enodes[q].z};
  return a;
}

// Reverse steps n_hi-1 … n_lo; the trace buffer holds steps from trace_n0. Whole pairs of
// K-step launches of the temporally blocked sweep first (when prepared), the rest one step
// per launch pair; both give the same bits.
template <typename T>
int backward_sweep(etg_adj* A, int64_t n_hi, int64_t n_lo, int64_t trace_n0, int* par_e, int* par_h,
                   const AdjPlan<T>& ph, const AdjPlan<T>& pe) {
  etg_sim* s = A->sim;
  const SimArgs<T> sa = sim_args_of<T>(s);
  int ER, EC, K;
  tb_adj_shape(s->dtype, &ER, &EC, &K);
  const int64_t pairs = A->tiles ? (n_hi - n_lo) / (2 * K) : 0;
  if (pairs) {  // K-step launch pairs, captured in graphs of per_graph pairs
    const int64_t ctl[2] = {n_hi, trace_n0};
    ETG_TRY_CUDA(cudaMemcpyAsync(A->d_ctl, ctl, sizeof ctl, cudaMemcpyHostToDevice, s->stream));
    const TBAdjArgs<T> to_alt = tb_adj_args<T>(A, sa, *par_e, *par_h, A->d_ctl, true);
    const TBAdjArgs<T> back = tb_adj_args<T>(A, sa, *par_e, *par_h, A->d_ctl, false);
    ETG_TRY_CUDA(cudaMemcpyAsync(A->d_args1, &to_alt, sizeof to_alt, cudaMemcpyHostToDevice, s->stream));
    const int64_t nodes = (int64_t)A->nxd * (A->nyd + 1) + (int64_t)(A->nxd + 1) * A->nyd;
    auto block_end = [&](int64_t n_pairs) {  // dJ/dcb of the block's steps, then the next block
      tb_adj_grad<T>((const TBAdjArgs<T>*)A->d_args1, 1, 1, nodes, (int)(2 * K * n_pairs), s->stream);
      tb_adj_ctl_add(A->d_ctl, -2 * K * n_pairs, s->stream);
    };
    auto pair = [&](int64_t p) {
      int rc = tb_adj_launch<T>(to_alt, A->tiles, A->n_inner, A->n_kind, (int)(2 * K * p), s->stream, A->sides,
                                A->fork, A->joins);
      if (rc == ETG_OK)
        rc = tb_adj_launch<T>(back, A->tiles, A->n_inner, A->n_kind, (int)(2 * K * p + K), s->stream, A->sides,
                              A->fork, A->joins);
      return rc;
    };
    const int64_t per_graph = std::max<int64_t>(1, s->opt[ETG_OPT_GRAPH_STEPS] / (2 * K));
    int64_t done = 0;
    if (s->opt[ETG_OPT_GRAPH_STEPS] > 0 && pairs >= per_graph) {
      const int64_t key = 2 * per_graph + *par_e;
      auto it = A->graphs.find(key);
      if (it == A->graphs.end()) {
        cudaGraph_t graph;
        ETG_TRY_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
        int rc = ETG_OK;
        for (int64_t p = 0; p < per_graph && rc == ETG_OK; ++p) rc = pair(p);
        if (rc == ETG_OK) block_end(per_graph);
        cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
        if (rc) return rc;
        ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "adjoint graph capture failed: %s", cudaGetErrorString(e));
        cudaGraphExec_t exec;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "adjoint graph instantiate failed: %s", cudaGetErrorString(e));
        it = A->graphs.emplace(key, exec).first;
      }
      for (; done + per_graph <= pairs; done += per_graph) {
        ETG_TRY_CUDA(cudaGraphLaunch(it->second, s->stream));
        g_launches += 4 * per_graph + 2;
      }
    }
    while (done < pairs) {  // without graphs, blocks of at most per_graph pairs
      const int64_t c = std::min(per_graph, pairs - done);
      for (int64_t p = 0; p < c; ++p) {
        int rc = pair(p);
        if (rc) return rc;
      }
      block_end(c);
      done += c;
    }
    n_hi -= 2 * K * pairs;
  }
  const dim3 block(32, 4);
  const dim3 gre((s->ny + 31) / 32, (s->nx + 3) / 4), grh((s->ny + 1 + 31) / 32, (s->nx + 1 + 3) / 4);
  for (int64_t n = n_hi - 1; n >= n_lo; --n) {
    AdjArgs<T> a = adj_args<T>(A, sa, *par_e, *par_h, trace_n0);
    k_adj_re<T><<<gre, block, 0, s->stream>>>(a, ph, n);
    *par_e ^= 1;
    a = adj_args<T>(A, sa, *par_e, *par_h, trace_n0);
    k_adj_rh<T><<<grh, block, 0, s->stream>>>(a, pe, n >= 1 ? n - 1 : -1);
    *par_h ^= 1;
    g_launches += 2;
  }
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

template <typename T>
int build_adj_plans(etg_adj* A, AdjPlan<T>* ph, AdjPlan<T>* pe) {
  memset(ph, 0, sizeof *ph);
  memset(pe, 0, sizeof *pe);
  etg_sim* s = A->sim;
  for (size_t k = 0; k < s->monitors.size(); ++k) {
    if (!A->gacc[k]) continue;
    const Monitor& m = s->monitors[k];
    AdjPlan<T>* p = m.comp == ETG_HZ ? ph : pe;
    ETG_REQUIRE(p->n_mon < MAX_MONITORS, ETG_ERR_ARGUMENT, "too many monitors in the objective");
    ETG_REQUIRE(m.n0 <= 0 && A->n_steps <= m.n0 + m.rows, ETG_ERR_STATE,
                "monitor %zu has phasors for steps [%lld, %lld), the adjoint needs [0, %lld)", k,
                (long long)m.n0, (long long)(m.n0 + m.rows), (long long)A->n_steps);
    AdjMon<T>& d = p->mon[p->n_mon++];
    d.table = (const T*)m.table;
    d.g = (const T*)A->gacc[k];
    d.n0 = m.n0;
    d.rows = m.rows;
    d.ix0 = m.ix0;
    d.nxm = m.nxm;
    d.jy0 = m.jy0;
    d.nym = m.nym;
    d.n_f = m.n_f;
    d.comp = m.comp;
  }
  return ETG_OK;
}

void drop_tb(etg_adj* A) {
  for (auto& kv : A->graphs) cudaGraphExecDestroy(kv.second);
  A->graphs.clear();
  for (void*& p : A->alt) {
    cudaFree(p);
    p = nullptr;
  }
  cudaFree(A->tiles);
  A->tiles = nullptr;
}

// The temporally blocked sweep, unless the simulation is pinned to the one-step kernels or
// the objective has more adjoint-source nodes than a launch carries: second lambda buffer,
// tiles (adjoint-source nodes and the design window lead), per-node source tables.
template <typename T>
int prepare_tb(etg_adj* A, const AdjPlan<T>& ph, const AdjPlan<T>& pe) {
  etg_sim* s = A->sim;
  for (auto& kv : A->graphs) cudaGraphExecDestroy(kv.second);  // arguments change every pass
  A->graphs.clear();
  A->hnodes.clear();
  A->enodes.clear();
  if (s->opt[ETG_OPT_KERNEL] == 1) {
    drop_tb(A);
    return ETG_OK;
  }
  auto collect = [](const AdjPlan<T>& p, std::vector<int4>* out) {
    for (int m = 0; m < p.n_mon; ++m) {
      const AdjMon<T>& d = p.mon[m];
      for (int a = 0; a < d.nxm; ++a)
        for (int b = 0; b < d.nym; ++b) {
          const int4 q = make_int4(d.ix0 + a, d.jy0 + b, d.comp, 0);
          bool seen = false;
          for (const int4& o : *out) seen |= o.x == q.x && o.y == q.y && o.z == q.z;
          if (!seen) out->push_back(q);
          if (out->size() > (size_t)MAX_SRC_NODES) return false;
        }
    }
    return true;
  };
  if (!collect(ph, &A->hnodes) || !collect(pe, &A->enodes)) {
    A->hnodes.clear();
    A->enodes.clear();
    drop_tb(A);
    return ETG_OK;  // too many source nodes: one-step sweep
  }
  int rc = tb_adj_attrs<T>();
  if (rc) return rc;
  if (!A->d_ctl) {
    rc = etg_malloc((void**)&A->d_ctl, 2 * sizeof(int64_t));
    if (rc) return rc;
  }
  if (!A->d_args1) {
    rc = etg_malloc(&A->d_args1, sizeof(TBAdjArgs<T>));
    if (rc) return rc;
  }
  {  // lambda E of the window for every step of the largest launch block (graph or batch)
    int ER, EC, K;
    tb_adj_shape(s->dtype, &ER, &EC, &K);
    const int64_t slots = 2 * K * std::max<int64_t>({1, s->opt[ETG_OPT_GRAPH_STEPS] / (2 * K), kBatchPairsPerGraph});
    if (slots > A->ltrace_slots) {
      cudaFree(A->ltrace);
      A->ltrace = nullptr;
      A->ltrace_slots = 0;
      rc = etg_malloc(&A->ltrace, (size_t)slots * 2 * (A->nxd + 1) * (A->nyd + 1) * sizeof(T));
      if (rc) return rc;
      A->ltrace_slots = slots;
    }
  }
  const size_t pb = plane_bytes(s);
  for (void*& p : A->alt) {  // kept from pass to pass; lambda psi must start at +0 in both buffers
    if (!p) {
      rc = etg_malloc(&p, pb);
      if (rc) return rc;
    }
    ETG_TRY_CUDA(cudaMemsetAsync(p, 0, pb, s->stream));
  }
  int ER, EC, K;
  tb_adj_shape(s->dtype, &ER, &EC, &K);
  std::vector<int4> hot;
  for (const int4& q : A->hnodes) hot.push_back(make_int4(q.x, q.y, q.x + 1, q.y + 1));
  for (const int4& q : A->enodes) hot.push_back(make_int4(q.x, q.y, q.x + 1, q.y + 1));
  hot.push_back(make_int4(A->i0, A->j0, A->i0 + A->nxd + 1, A->j0 + A->nyd + 1));
  std::vector<int2> tiles;
  tb_split_tiles(s->nx, s->ny, s->ux_lo, s->ux_hi, s->uy_lo, s->uy_hi, ER, EC, K, hot, &tiles, &A->n_inner);
  A->n_pml = (int)tiles.size() - A->n_inner;
  for (int k = 0; k < 3; ++k) A->n_kind[k] = 0;
  for (int q = A->n_inner; q < (int)tiles.size(); ++q) A->n_kind[tb_tile_kind(tiles[q]) - 1] += 1;
  if (!A->tiles || tiles.size() != A->h_tiles.size() ||
      memcmp(tiles.data(), A->h_tiles.data(), tiles.size() * sizeof(int2)) != 0) {
    cudaFree(A->tiles);
    A->tiles = nullptr;
    rc = etg_malloc((void**)&A->tiles, tiles.size() * sizeof(int2));
    if (rc) return rc;
    ETG_TRY_CUDA(cudaMemcpy(A->tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice));
    A->h_tiles = tiles;
  }
  // adjoint-source tables: H nodes from the H plan, E nodes from the E plan
  const int64_t N = A->n_steps;
  const size_t bytes = std::max<size_t>(1, (A->hnodes.size() + A->enodes.size()) * N * sizeof(T));
  if (A->tables_bytes < bytes) {
    cudaFree(A->tables);
    A->tables = nullptr;
    A->tables_bytes = 0;
    rc = etg_malloc(&A->tables, bytes);
    if (rc) return rc;
    A->tables_bytes = bytes;
  }
  for (int which = 0; which < 2; ++which) {
    const std::vector<int4>& nodes = which == 0 ? A->hnodes : A->enodes;
    if (nodes.empty()) continue;
    int4* d_nodes = nullptr;
    rc = etg_malloc((void**)&d_nodes, nodes.size() * sizeof(int4));
    if (rc) return rc;
    ETG_TRY_CUDA(cudaMemcpy(d_nodes, nodes.data(), nodes.size() * sizeof(int4), cudaMemcpyHostToDevice));
    T* out = (T*)A->tables + (which == 0 ? 0 : A->hnodes.size() * N);
    const int64_t total = (int64_t)nodes.size() * N;
    k_adj_tables<T><<<(unsigned)((total + 255) / 256), 256, 0, s->stream>>>(which == 0 ? ph : pe, d_nodes,
                                                                           (int)nodes.size(), N, out);
    g_launches += 1;
    cudaError_t e = cudaStreamSynchronize(s->stream);
    cudaFree(d_nodes);
    ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "adjoint source tables: %s", cudaGetErrorString(e));
  }
  if (!A->side) {
    ETG_TRY_CUDA(cudaStreamCreateWithFlags(&A->side, cudaStreamNonBlocking));
    ETG_TRY_CUDA(cudaEventCreateWithFlags(&A->fork, cudaEventDisableTiming));
    ETG_TRY_CUDA(cudaEventCreateWithFlags(&A->join, cudaEventDisableTiming));
    for (int k = 0; k < 3; ++k) {
      ETG_TRY_CUDA(cudaStreamCreateWithFlags(&A->sides[k], cudaStreamNonBlocking));
      ETG_TRY_CUDA(cudaEventCreateWithFlags(&A->joins[k], cudaEventDisableTiming));
    }
  }
  return ETG_OK;
}

// dJ/dacc of every monitor (nullptr: not in the objective), kept on the device.
int adj_set_objective(etg_adj* A, const void* const* grad_acc) {
  etg_sim* s = A->sim;
  for (void*& p : A->gacc) {
    cudaFree(p);
    p = nullptr;
  }
  A->gacc.assign(s->monitors.size(), nullptr);
  for (size_t k = 0; k < s->monitors.size(); ++k) {
    if (!grad_acc || !grad_acc[k]) continue;
    const Monitor& m = s->monitors[k];
    const size_t bytes = (size_t)2 * m.n_f * m.nxm * m.nym * s->esize();
    int rc = etg_malloc(&A->gacc[k], bytes);
    if (rc) return rc;
    ETG_TRY_CUDA(cudaMemcpy(A->gacc[k], grad_acc[k], bytes, cudaMemcpyHostToDevice));
  }
  return ETG_OK;
}

// Zero lambda and dJ/dcb, build the adjoint plans, prepare the blocked sweep and add the
// DFT-E source of the last step; lambda psi parities start at 0.
template <typename T>
int adj_begin(etg_adj* A, AdjPlan<T>* ph, AdjPlan<T>* pe) {
  etg_sim* s = A->sim;
  ETG_REQUIRE(A->n_steps > 0, ETG_ERR_STATE, "adjoint: run the forward pass first");
  const size_t pb = plane_bytes(s);
  for (int k = 0; k < 3; ++k) {
    int rc = ensure(&A->lam[k], pb);
    if (rc) return rc;
    ETG_TRY_CUDA(cudaMemsetAsync(A->lam[k], 0, pb, s->stream));
  }
  for (int b = 0; b < 2; ++b)
    for (int k = 0; k < 4; ++k) {
      int rc = ensure(&A->lpsi[b][k], pb);
      if (rc) return rc;
      ETG_TRY_CUDA(cudaMemsetAsync(A->lpsi[b][k], 0, pb, s->stream));
    }
  const size_t gbytes = ((size_t)A->nxd * (A->nyd + 1) + (size_t)(A->nxd + 1) * A->nyd) * sizeof(double);
  int rc = ensure((void**)&A->grad, gbytes);
  if (rc) return rc;
  ETG_TRY_CUDA(cudaMemsetAsync(A->grad, 0, gbytes, s->stream));
  if (A->gacc.size() != s->monitors.size()) A->gacc.assign(s->monitors.size(), nullptr);
  rc = build_adj_plans<T>(A, ph, pe);
  if (rc == ETG_OK) rc = prepare_tb<T>(A, *ph, *pe);
  if (rc) return rc;
  const SimArgs<T> sa = sim_args_of<T>(s);
  AdjArgs<T> a0 = adj_args<T>(A, sa, 0, 0, 0);
  const dim3 block(32, 4), grh((s->ny + 1 + 31) / 32, (s->nx + 1 + 3) / 4);
  k_adj_esrc<T><<<grh, block, 0, s->stream>>>(a0, *pe, A->n_steps - 1);
  g_launches += 1;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

// While segments of S steps are recomputed, only the light cone of the window's trace box is
// stepped: a value moves at most one cell per time step, so the trace box stays exact for S
// steps when every cell within S cells of it is, and the tiles beyond (their halos read cells
// that are not updated) only spoil cells farther out. The margin adds room for two launches
// of the deepest tiles. Checkpoints keep only that rectangle of the planes (one more row and
// column on each side, columns from a multiple of 4): nothing else is ever restored.
void cone_of(const etg_adj* A, int64_t S, int* i0, int* i1, int* j0, int* j1) {
  const int64_t m = S + 2 * 8 + 2;
  *i0 = (int)std::max<int64_t>(0, A->ti0 - m);
  *i1 = (int)std::min<int64_t>(1 << 30, A->ti0 + A->tnx + m);
  *j0 = (int)std::max<int64_t>(0, A->tj0 - m);
  *j1 = (int)std::min<int64_t>(1 << 30, A->tj0 + A->tny + m);
}

void set_cone(etg_adj* A, int64_t S) {
  etg_sim* s = A->sim;
  cone_of(A, S, &s->act_i0, &s->act_i1, &s->act_j0, &s->act_j1);
}

void clear_cone(etg_sim* s) {
  s->act_i0 = s->act_j0 = 0;
  s->act_i1 = s->act_j1 = 1 << 30;
}

// The checkpoint rectangle of A for segments of S steps.
void set_ckpt_rect(etg_adj* A, int64_t S) {
  const etg_sim* s = A->sim;
  int i0, i1, j0, j1;
  cone_of(A, S, &i0, &i1, &j0, &j1);
  A->ck_r0 = std::max(0, i0 - 1);
  A->ck_r1 = std::min<int64_t>(s->rows, (int64_t)i1 + 1);
  A->ck_c0 = std::max(0, j0 - 1) / 4 * 4;
  A->ck_c1 = std::min<int64_t>(s->P, (int64_t)j1 + 1);
}

size_t ckpt_bytes(const etg_adj* A) {
  return 7 * (size_t)std::max<int64_t>(0, A->ck_r1 - A->ck_r0) * std::max<int64_t>(0, A->ck_c1 - A->ck_c0) *
         A->sim->esize();
}

// The 7 plane copies of design A: fields -> checkpoint k (save) or checkpoint k -> fields,
// which also sets the step counter (restore).
void ckpt_copies(const etg_adj* A, bool save, std::vector<RectCopy>* out) {
  const etg_sim* s = A->sim;
  const int64_t es = (int64_t)s->esize(), rows = std::max<int64_t>(0, A->ck_r1 - A->ck_r0);
  const int64_t words = std::max<int64_t>(0, A->ck_c1 - A->ck_c0) * es / 4, plane = rows * words;
  for (int f = 0; f < 7; ++f) {
    uint32_t* field = (uint32_t*)((char*)s->field[f] + (A->ck_r0 * s->P + A->ck_c0) * es);
    uint32_t* ck = (uint32_t*)A->ckpt + f * plane;
    RectCopy c;
    c.src = save ? field : ck;
    c.dst = save ? ck : field;
    c.src_pitch = save ? s->P * es / 4 : words;
    c.dst_pitch = save ? words : s->P * es / 4;
    c.src_k = save ? 0 : 7 * plane;
    c.dst_k = save ? 7 * plane : 0;
    c.step = !save && f == 0 ? s->d_step : nullptr;
    c.rows = (int)rows;
    c.words = (int)words;
    out->push_back(c);
  }
}

// Upload a copy list (once per pass) and run it for checkpoint k in one launch.
int upload_copies(void** buf, size_t* cap, const std::vector<RectCopy>& copies, cudaStream_t st) {
  const size_t bytes = copies.size() * sizeof(RectCopy);
  if (*cap < bytes) {
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    int rc = etg_malloc(buf, bytes);
    if (rc) return rc;
    *cap = bytes;
  }
  ETG_TRY_CUDA(cudaMemcpyAsync(*buf, copies.data(), bytes, cudaMemcpyHostToDevice, st));
  return ETG_OK;
}

int run_copies(const void* buf, int n, int64_t k, int64_t step_value, cudaStream_t st) {
  k_copy_rects<<<dim3(64, (unsigned)n), 256, 0, st>>>((const RectCopy*)buf, k, step_value);
  g_launches += 1;
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

// Host side of restoring segment [lo, hi) of design A (the copies run separately): step
// index, and the trace it re-records.
void begin_segment(etg_adj* A, int64_t lo, int64_t hi) {
  A->sim->h_step = lo;
  A->sim->trace_cone = true;
  set_trace(A->sim, A->trace, lo, hi - lo, A);
}

template <typename T>
int adj_backward(etg_adj* A) {
  etg_sim* s = A->sim;
  AdjPlan<T> ph, pe;
  int rc = adj_begin<T>(A, &ph, &pe);
  if (rc) return rc;
  int par_e = 0, par_h = 0;
  if (A->stride == 0) {
    rc = backward_sweep<T>(A, A->n_steps, 0, 0, &par_e, &par_h, ph, pe);
  } else {
    const int64_t S = A->stride;
    const int64_t nseg = (A->n_steps + S - 1) / S;
    s->monitors_on = false;
    sim_invalidate(s);
    // the blocked path recomputes through a one-simulation batch, whose plans live in device
    // memory: moving the trace origin per segment then needs no new graphs
    if (A->tiles && !A->fwd1) {
      rc = etg_batch_create(&A->fwd1, 1, &s);
      // the light cone is a few dozen tiles, one wave on a fraction of the SMs: there a tile's
      // latency sets the time, and 16 warps of 3 rows hide it better than 8 warps (float32)
      if (rc == ETG_OK && s->dtype == ETG_F32 && s->opt[ETG_OPT_TB_WARPS] == 0 && s->opt[ETG_OPT_TILE_ROWS] == 0) {
        etg_batch_set_option(A->fwd1, ETG_OPT_TILE_ROWS, 48);
        etg_batch_set_option(A->fwd1, ETG_OPT_TB_WARPS, 16);
      }
    }
    set_cone(A, S);
    std::vector<RectCopy> copies;
    ckpt_copies(A, false, &copies);
    if (rc == ETG_OK) rc = upload_copies(&A->d_copies, &A->copies_cap, copies, s->stream);
    for (int64_t k = nseg - 1; k >= 0 && rc == ETG_OK; --k) {
      const int64_t lo = k * S, hi = std::min(A->n_steps, lo + S);
      rc = run_copies(A->d_copies, (int)copies.size(), k, lo, s->stream);
      begin_segment(A, lo, hi);
      if (rc == ETG_OK) {
        if (A->tiles) {  // the simulation's stream (the sweep's) waits for the recompute
          rc = etg_batch_advance(A->fwd1, hi - lo);
        } else {
          rc = sim_advance_internal(s, hi - lo);
        }
      }
      clear_trace(s);
      if (rc == ETG_OK) rc = backward_sweep<T>(A, hi, lo, lo, &par_e, &par_h, ph, pe);
    }
    clear_cone(s);
    s->monitors_on = true;
    sim_invalidate(s);
    if (rc == ETG_OK && A->fwd1) rc = etg_batch_synchronize(A->fwd1);  // device flags of the recomputes
  }
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return rc;
}

int adj_download(etg_adj* A, double* gx_host, double* gy_host) {
  ETG_REQUIRE(A->grad, ETG_ERR_STATE, "adjoint: no gradient yet, run the backward pass first");
  ETG_TRY_CUDA(cudaMemcpy(gx_host, A->grad, (size_t)A->nxd * (A->nyd + 1) * sizeof(double), cudaMemcpyDeviceToHost));
  ETG_TRY_CUDA(cudaMemcpy(gy_host, A->grad + (size_t)A->nxd * (A->nyd + 1),
                          (size_t)(A->nxd + 1) * A->nyd * sizeof(double), cudaMemcpyDeviceToHost));
  return ETG_OK;
}

// Forward pass recording what the gradient needs: the Hz trace of every step (stride 0) or
// full-state checkpoints every `stride` steps. Resets the simulation first.
int adj_forward_setup(etg_adj* A, int64_t n_steps, int64_t stride) {
  etg_sim* s = A->sim;
  int rc = etg_sim_reset(s);
  if (rc) return rc;
  A->n_steps = n_steps;
  A->stride = stride;
  const size_t cell_bytes = (size_t)A->tnx * A->tny * s->esize();
  const int64_t rows = stride == 0 ? n_steps : std::min(stride, n_steps);
  if (A->trace_cap < rows * cell_bytes) {
    cudaFree(A->trace);
    A->trace = nullptr;
    A->trace_cap = 0;
    rc = etg_malloc(&A->trace, rows * cell_bytes);
    if (rc) return rc;
    A->trace_cap = rows * cell_bytes;
  }
  if (stride > 0) {
    const int64_t nseg = (n_steps + stride - 1) / stride;
    set_ckpt_rect(A, stride);
    const size_t bytes = std::max<size_t>(1, (size_t)nseg * ckpt_bytes(A));
    if (A->ckpt_cap < bytes) {
      cudaFree(A->ckpt);
      A->ckpt = nullptr;
      A->ckpt_cap = 0;
      rc = etg_malloc(&A->ckpt, bytes);
      if (rc) return rc;
      A->ckpt_cap = bytes;
    }
  }
  return ETG_OK;
}

// ------------------------------------------------------------------ many designs at once

}  // namespace

struct etg_adj_batch {
  std::vector<etg_adj*> adjs;
  int dtype = ETG_F32;
  etg_batch* fwd = nullptr;  // the simulations stepped together
  void* d_args = nullptr;    // TBAdjArgs<T>[2 n]: reading the primary / the second lambda buffer
  int4* d_tiles = nullptr;
  int n_inner = 0, n_pml = 0;
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaEvent_t seg_done = nullptr;  // a segment's recompute is done
  void* d_copies = nullptr;        // RectCopy list of every design's checkpoint save or restore
  size_t copies_cap = 0;
  cudaStream_t sides[3] = {};  // one branch per CPML kind
  cudaEvent_t joins[3] = {};
  int n_kind[3] = {};
  int64_t n_steps = 0, stride = 0;
  int64_t* d_ctl = nullptr;                   // top step of the launch block, trace origin
  std::map<int64_t, cudaGraphExec_t> graphs;  // key: pairs per graph
};

namespace {

// Batched reverse steps n_hi-1 … n_lo of every design: whole K-step launch pairs over the
// tiles of all designs, then each design's remainder with the one-step kernels.
template <typename T>
int batch_sweep(etg_adj_batch* B, int64_t n_hi, int64_t n_lo, int64_t trace_n0, std::vector<int>& par_e,
                std::vector<int>& par_h, const std::vector<AdjPlan<T>>& ph, const std::vector<AdjPlan<T>>& pe) {
  const int n = (int)B->adjs.size();
  int ER, EC, K;
  tb_adj_shape(B->dtype, &ER, &EC, &K);
  const int64_t pairs = B->d_tiles ? (n_hi - n_lo) / (2 * K) : 0;
  if (pairs) {
    std::vector<TBAdjArgs<T>> args(2 * n);
    for (int k = 0; k < n; ++k) {
      etg_adj* A = B->adjs[k];
      const SimArgs<T> sa = sim_args_of<T>(A->sim);
      args[2 * k] = tb_adj_args<T>(A, sa, par_e[k], par_h[k], B->d_ctl, true);
      args[2 * k + 1] = tb_adj_args<T>(A, sa, par_e[k], par_h[k], B->d_ctl, false);
      ETG_TRY_CUDA(cudaStreamSynchronize(A->sim->stream));
    }
    const int64_t ctl[2] = {n_hi, trace_n0};
    ETG_TRY_CUDA(cudaMemcpyAsync(B->d_ctl, ctl, sizeof ctl, cudaMemcpyHostToDevice, B->stream));
    ETG_TRY_CUDA(cudaMemcpyAsync(B->d_args, args.data(), args.size() * sizeof(TBAdjArgs<T>), cudaMemcpyHostToDevice,
                                 B->stream));
    const TBAdjArgs<T>* d_args = (const TBAdjArgs<T>*)B->d_args;
    int64_t max_nodes = 0;
    for (const etg_adj* A : B->adjs)
      max_nodes = std::max<int64_t>(max_nodes, (int64_t)A->nxd * (A->nyd + 1) + (int64_t)(A->nxd + 1) * A->nyd);
    auto block_end = [&](int64_t n_pairs) {
      tb_adj_grad<T>(d_args, 2, n, max_nodes, (int)(2 * K * n_pairs), B->stream);
      tb_adj_ctl_add(B->d_ctl, -2 * K * n_pairs, B->stream);
    };
    auto pair = [&](int64_t p) {
      int rc = tb_adj_batch_launch<T>(d_args, B->d_tiles, B->n_inner, B->n_kind, 0, (int)(2 * K * p), B->stream,
                                      B->sides, B->fork, B->joins);
      if (rc == ETG_OK)
        rc = tb_adj_batch_launch<T>(d_args, B->d_tiles, B->n_inner, B->n_kind, 1, (int)(2 * K * p + K), B->stream,
                                    B->sides, B->fork, B->joins);
      return rc;
    };
    const int64_t per_graph = kBatchPairsPerGraph;
    int64_t done = 0;
    if (pairs >= per_graph) {
      auto it = B->graphs.find(per_graph);
      if (it == B->graphs.end()) {
        cudaGraph_t graph;
        ETG_TRY_CUDA(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
        int rc = ETG_OK;
        for (int64_t p = 0; p < per_graph && rc == ETG_OK; ++p) rc = pair(p);
        if (rc == ETG_OK) block_end(per_graph);
        cudaError_t e = cudaStreamEndCapture(B->stream, &graph);
        if (rc) return rc;
        ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "batched adjoint graph capture failed: %s", cudaGetErrorString(e));
        cudaGraphExec_t exec;
        e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "batched adjoint graph instantiate failed: %s",
                    cudaGetErrorString(e));
        it = B->graphs.emplace(per_graph, exec).first;
      }
      for (; done + per_graph <= pairs; done += per_graph) {
        ETG_TRY_CUDA(cudaGraphLaunch(it->second, B->stream));
        g_launches += 4 * per_graph + 2;
      }
    }
    if (done < pairs) {
      for (int64_t p = 0; done + p < pairs; ++p) {
        int rc = pair(p);
        if (rc) return rc;
      }
      block_end(pairs - done);
    }
    ETG_TRY_CUDA(cudaStreamSynchronize(B->stream));  // the host copy of args stays alive until here
  }
  const int64_t top = n_hi - 2 * K * pairs;
  for (int k = 0; k < n && top > n_lo; ++k) {
    int rc = backward_sweep<T>(B->adjs[k], top, n_lo, trace_n0, &par_e[k], &par_h[k], ph[k], pe[k]);
    if (rc) return rc;
  }
  for (etg_adj* A : B->adjs) ETG_TRY_CUDA(cudaStreamSynchronize(A->sim->stream));
  return ETG_OK;
}

template <typename T>
int batch_backward(etg_adj_batch* B) {
  const int n = (int)B->adjs.size();
  std::vector<AdjPlan<T>> ph(n), pe(n);
  bool blocked = true;
  for (int k = 0; k < n; ++k) {
    int rc = adj_begin<T>(B->adjs[k], &ph[k], &pe[k]);
    if (rc) return rc;
    blocked &= B->adjs[k]->tiles != nullptr;
  }
  // one tile list over all designs, interior tiles first (graphs hold its address)
  for (auto& kv : B->graphs) cudaGraphExecDestroy(kv.second);
  B->graphs.clear();
  cudaFree(B->d_tiles);
  B->d_tiles = nullptr;
  if (!B->d_ctl) {
    int rc = etg_malloc((void**)&B->d_ctl, 2 * sizeof(int64_t));
    if (rc) return rc;
  }
  if (blocked) {
    std::vector<int4> inner, pml;
    for (int k = 0; k < n; ++k) {
      const etg_adj* A = B->adjs[k];
      for (int q = 0; q < (int)A->h_tiles.size(); ++q)
        (q < A->n_inner ? inner : pml)
            .push_back(make_int4(k, tb_tile_row(A->h_tiles[q]), A->h_tiles[q].y, tb_tile_kind(A->h_tiles[q])));
    }
    std::stable_sort(pml.begin(), pml.end(), [](const int4& p, const int4& q) { return p.w < q.w; });
    for (int k = 0; k < 3; ++k) B->n_kind[k] = 0;
    for (const int4& q : pml) B->n_kind[q.w - 1] += 1;
    B->n_inner = (int)inner.size();
    B->n_pml = (int)pml.size();
    inner.insert(inner.end(), pml.begin(), pml.end());
    int rc = etg_malloc((void**)&B->d_tiles, inner.size() * sizeof(int4));
    if (rc) return rc;
    ETG_TRY_CUDA(cudaMemcpy(B->d_tiles, inner.data(), inner.size() * sizeof(int4), cudaMemcpyHostToDevice));
    if (!B->d_args) {
      rc = etg_malloc(&B->d_args, 2 * n * sizeof(TBAdjArgs<T>));
      if (rc) return rc;
    }
  }
  std::vector<int> par_e(n, 0), par_h(n, 0);
  if (B->stride == 0) return batch_sweep<T>(B, B->n_steps, 0, 0, par_e, par_h, ph, pe);
  const int64_t S = B->stride;
  const int64_t nseg = (B->n_steps + S - 1) / S;
  for (etg_adj* A : B->adjs) {
    A->sim->monitors_on = false;
    set_cone(A, S);
    sim_invalidate(A->sim);
  }
  // one launch restores every design's light cone and step counter; the batch then waits for
  // it (it synchronises the simulations' streams first)
  std::vector<RectCopy> copies;
  for (etg_adj* A : B->adjs) ckpt_copies(A, false, &copies);
  cudaStream_t cs = B->adjs[0]->sim->stream;
  int rc = upload_copies(&B->d_copies, &B->copies_cap, copies, cs);
  for (int64_t k = nseg - 1; k >= 0 && rc == ETG_OK; --k) {
    const int64_t lo = k * S, hi = std::min(B->n_steps, lo + S);
    rc = run_copies(B->d_copies, (int)copies.size(), k, lo, cs);
    for (etg_adj* A : B->adjs) begin_segment(A, lo, hi);
    if (rc == ETG_OK) rc = etg_batch_advance(B->fwd, hi - lo);
    if (rc == ETG_OK) {  // the sweep's stream waits for the recompute (the simulations' streams wait for it)
      cudaError_t e = cudaEventRecord(B->seg_done, B->adjs[0]->sim->stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(B->stream, B->seg_done, 0);
      ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "adjoint batch: %s", cudaGetErrorString(e));
    }
    for (etg_adj* A : B->adjs) clear_trace(A->sim);
    if (rc == ETG_OK) rc = batch_sweep<T>(B, hi, lo, lo, par_e, par_h, ph, pe);
  }
  for (etg_adj* A : B->adjs) {
    clear_cone(A->sim);
    A->sim->monitors_on = true;
    sim_invalidate(A->sim);
  }
  if (rc == ETG_OK) rc = etg_batch_synchronize(B->fwd);  // device flags of the recomputes
  return rc;
}

}  // namespace

extern "C" {

int etg_adj_create(etg_adj** out, etg_sim* sim, int i0, int nxd, int j0, int nyd) {
  ETG_REQUIRE(out && sim, ETG_ERR_ARGUMENT, "etg_adj_create: null argument");
  ETG_REQUIRE(nxd > 0 && nyd > 0, ETG_ERR_ARGUMENT, "etg_adj_create: empty design window");
  ETG_REQUIRE(!sim->db_node, ETG_ERR_ARGUMENT,
              "etg_adj_create: the adjoint is for TE runs; this simulation has per-node Hz coefficients (TM mode)");
  // the window with one cell of halo must lie in the unit rectangle, off the PEC edges
  const int rlo = std::max(sim->ux_lo, 1), rhi = std::min(sim->ux_hi, sim->nx);
  const int clo = std::max(sim->uy_lo, 1), chi = std::min(sim->uy_hi, sim->ny);
  ETG_REQUIRE(i0 - 1 >= rlo && i0 + nxd + 1 <= rhi && j0 - 1 >= clo && j0 + nyd + 1 <= chi,
              ETG_ERR_ARGUMENT,
              "etg_adj_create: design window [%d,%d)x[%d,%d) must lie, with one cell of margin, inside "
              "the region where the CPML terms vanish ([%d,%d)x[%d,%d))",
              i0, i0 + nxd, j0, j0 + nyd, rlo, rhi, clo, chi);
  for (const Source& src : sim->sources)
    for (size_t k = 0; k < src.i.size(); ++k)
      ETG_REQUIRE(src.comp == ETG_HZ || !(src.i[k] >= i0 - 1 && src.i[k] <= i0 + nxd && src.j[k] >= j0 - 1 &&
                                          src.j[k] <= j0 + nyd),
                  ETG_ERR_ARGUMENT, "etg_adj_create: an electric source lies on the design window");
  etg_adj* A = new etg_adj;
  A->sim = sim;
  A->i0 = i0;
  A->nxd = nxd;
  A->j0 = j0;
  A->nyd = nyd;
  A->ti0 = i0 - 1;
  A->tnx = nxd + 2;
  A->tj0 = j0 - 1;
  A->tny = nyd + 2;
  *out = A;
  return ETG_OK;
}

int etg_adj_destroy(etg_adj* A) {
  if (!A) return ETG_OK;
  if (A->sim && A->sim->trace_buf == A->trace) clear_trace(A->sim);
  cudaFree(A->trace);
  cudaFree(A->ckpt);
  cudaFree(A->d_copies);
  for (void* p : A->lam) cudaFree(p);
  for (auto& b : A->lpsi)
    for (void* p : b) cudaFree(p);
  cudaFree(A->grad);
  for (void* p : A->gacc) cudaFree(p);
  drop_tb(A);
  etg_batch_destroy(A->fwd1);
  cudaFree(A->d_ctl);
  cudaFree(A->ltrace);
  cudaFree(A->d_args1);
  cudaFree(A->tables);
  if (A->fork) cudaEventDestroy(A->fork);
  if (A->join) cudaEventDestroy(A->join);
  if (A->side) cudaStreamDestroy(A->side);
  for (int k = 0; k < 3; ++k) {
    if (A->sides[k]) cudaStreamDestroy(A->sides[k]);
    if (A->joins[k]) cudaEventDestroy(A->joins[k]);
  }
  delete A;
  return ETG_OK;
}

int etg_adj_forward(etg_adj* A, int64_t n_steps, int64_t stride) {
  ETG_REQUIRE(A && n_steps > 0 && stride >= 0, ETG_ERR_ARGUMENT, "etg_adj_forward: bad arguments");
  etg_sim* s = A->sim;
  int rc = adj_forward_setup(A, n_steps, stride);
  if (rc) return rc;
  if (stride == 0) {
    set_trace(s, A->trace, 0, n_steps, A);
    rc = sim_advance_internal(s, n_steps);
    clear_trace(s);
    if (rc) return rc;
  } else {
    std::vector<RectCopy> copies;
    ckpt_copies(A, true, &copies);
    rc = upload_copies(&A->d_copies, &A->copies_cap, copies, s->stream);
    const int64_t nseg = (n_steps + stride - 1) / stride;
    for (int64_t k = 0; k < nseg && rc == ETG_OK; ++k) {
      rc = run_copies(A->d_copies, (int)copies.size(), k, -1, s->stream);
      if (rc == ETG_OK) rc = sim_advance_internal(s, std::min(stride, n_steps - k * stride));
    }
    if (rc) return rc;
  }
  return etg_sim_synchronize(s);
}

int etg_adj_set_objective(etg_adj* A, const void* const* grad_acc) {
  ETG_REQUIRE(A, ETG_ERR_ARGUMENT, "etg_adj_set_objective: null handle");
  return adj_set_objective(A, grad_acc);
}

int etg_adj_gradient(etg_adj* A, double* grad_cb_ex, double* grad_cb_ey) {
  ETG_REQUIRE(A && grad_cb_ex && grad_cb_ey, ETG_ERR_ARGUMENT, "etg_adj_gradient: null argument");
  return adj_download(A, grad_cb_ex, grad_cb_ey);
}

int etg_adj_backward(etg_adj* A, const void* const* grad_acc, double* grad_cb_ex, double* grad_cb_ey) {
  ETG_REQUIRE(A && grad_cb_ex && grad_cb_ey, ETG_ERR_ARGUMENT, "etg_adj_backward: null argument");
  ETG_REQUIRE(A->n_steps > 0, ETG_ERR_STATE, "etg_adj_backward: run etg_adj_forward first");
  int rc = adj_set_objective(A, grad_acc);
  if (rc) return rc;
  rc = A->sim->dtype == ETG_F32 ? adj_backward<float>(A) : adj_backward<double>(A);
  if (rc) return rc;
  rc = etg_sim_synchronize(A->sim);
  if (rc) return rc;
  return adj_download(A, grad_cb_ex, grad_cb_ey);
}

int etg_adj_batch_create(etg_adj_batch** out, int n, etg_adj* const* adjs) {
  ETG_REQUIRE(out && adjs && n > 0, ETG_ERR_ARGUMENT, "etg_adj_batch_create: bad arguments");
  std::vector<etg_sim*> sims(n);
  for (int k = 0; k < n; ++k) {
    ETG_REQUIRE(adjs[k], ETG_ERR_ARGUMENT, "etg_adj_batch_create: design %d is null", k);
    ETG_REQUIRE(adjs[k]->sim->dtype == adjs[0]->sim->dtype, ETG_ERR_ARGUMENT, "etg_adj_batch_create: mixed precisions");
    for (int q = 0; q < k; ++q)
      ETG_REQUIRE(adjs[q]->sim != adjs[k]->sim, ETG_ERR_ARGUMENT, "etg_adj_batch_create: designs %d and %d share a simulation", q, k);
    sims[k] = adjs[k]->sim;
  }
  etg_adj_batch* B = new etg_adj_batch;
  B->adjs.assign(adjs, adjs + n);
  B->dtype = adjs[0]->sim->dtype;
  int rc = etg_batch_create(&B->fwd, n, sims.data());
  if (rc == ETG_OK &&
      (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->join, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->seg_done, cudaEventDisableTiming) != cudaSuccess ||
       cudaStreamCreateWithFlags(&B->sides[0], cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&B->sides[1], cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&B->sides[2], cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->joins[0], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->joins[1], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&B->joins[2], cudaEventDisableTiming) != cudaSuccess)) {
    set_error("etg_adj_batch_create: %s", cudaGetErrorString(cudaGetLastError()));
    rc = ETG_ERR_CUDA;
  }
  if (rc) {
    etg_adj_batch_destroy(B);
    return rc;
  }
  *out = B;
  return ETG_OK;
}

int etg_adj_batch_destroy(etg_adj_batch* B) {
  if (!B) return ETG_OK;
  if (B->stream) cudaStreamSynchronize(B->stream);
  etg_batch_destroy(B->fwd);
  for (auto& kv : B->graphs) cudaGraphExecDestroy(kv.second);
  cudaFree(B->d_ctl);
  cudaFree(B->d_args);
  cudaFree(B->d_tiles);
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->join) cudaEventDestroy(B->join);
  if (B->seg_done) cudaEventDestroy(B->seg_done);
  cudaFree(B->d_copies);
  if (B->side) cudaStreamDestroy(B->side);
  for (int k = 0; k < 3; ++k) {
    if (B->sides[k]) cudaStreamDestroy(B->sides[k]);
    if (B->joins[k]) cudaEventDestroy(B->joins[k]);
  }
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
  return ETG_OK;
}

int etg_adj_batch_set_option(etg_adj_batch* B, int option, int64_t value) {
  ETG_REQUIRE(B, ETG_ERR_ARGUMENT, "etg_adj_batch_set_option: null handle");
  return etg_batch_set_option(B->fwd, option, value);
}

int etg_adj_batch_forward(etg_adj_batch* B, int64_t n_steps, int64_t stride) {
  ETG_REQUIRE(B && n_steps > 0 && stride >= 0, ETG_ERR_ARGUMENT, "etg_adj_batch_forward: bad arguments");
  for (etg_adj* A : B->adjs) {
    int rc = adj_forward_setup(A, n_steps, stride);
    if (rc) return rc;
  }
  B->n_steps = n_steps;
  B->stride = stride;
  int rc = ETG_OK;
  if (stride == 0) {
    for (etg_adj* A : B->adjs) set_trace(A->sim, A->trace, 0, n_steps, A);
    rc = etg_batch_advance(B->fwd, n_steps);
    if (rc == ETG_OK) rc = etg_batch_synchronize(B->fwd);
    for (etg_adj* A : B->adjs) clear_trace(A->sim);
    return rc;
  }
  // one launch saves every design's checkpoint k (the batch makes every simulation's stream
  // wait for its steps, and synchronises them before the next ones)
  std::vector<RectCopy> copies;
  for (etg_adj* A : B->adjs) ckpt_copies(A, true, &copies);
  cudaStream_t cs = B->adjs[0]->sim->stream;
  rc = upload_copies(&B->d_copies, &B->copies_cap, copies, cs);
  const int64_t nseg = (n_steps + stride - 1) / stride;
  for (int64_t k = 0; k < nseg && rc == ETG_OK; ++k) {
    rc = run_copies(B->d_copies, (int)copies.size(), k, -1, cs);
    if (rc == ETG_OK) rc = etg_batch_advance(B->fwd, std::min(stride, n_steps - k * stride));
  }
  if (rc == ETG_OK) rc = etg_batch_synchronize(B->fwd);
  return rc;
}

int etg_adj_batch_backward(etg_adj_batch* B) {
  ETG_REQUIRE(B, ETG_ERR_ARGUMENT, "etg_adj_batch_backward: null handle");
  ETG_REQUIRE(B->n_steps > 0, ETG_ERR_STATE, "etg_adj_batch_backward: run etg_adj_batch_forward first");
  for (etg_adj* A : B->adjs)
    ETG_REQUIRE(A->n_steps == B->n_steps && A->stride == B->stride, ETG_ERR_STATE,
                "etg_adj_batch_backward: a design was run on its own since the batched forward pass");
  int rc = B->dtype == ETG_F32 ? batch_backward<float>(B) : batch_backward<double>(B);
  if (rc) return rc;
  for (etg_adj* A : B->adjs) {
    rc = etg_sim_synchronize(A->sim);
    if (rc) return rc;
  }
  return ETG_OK;
}

}  // extern "C"
