// Temporally blocked reverse sweep of the discrete adjoint (K reverse steps per launch).
#pragma once

#include "etg_sim.h"

namespace etg {

// One adjoint source node: lambda(comp at i, j) += table[n] at reverse step n (H nodes) or
// table[n - 1] (E nodes, the DFT-E term of step n - 1). The table holds, for every step, the
// sum over the objective's monitors of Re(G)·Re(ph) + Im(G)·Im(ph) in the order the one-step
// adjoint kernel adds them.
template <typename T>
struct AdjSrc {
  const T* table;
  int i, j, comp;
};

// Everything one temporally blocked adjoint launch reads and writes. Lambda planes are
// pitched like the fields: in/out[0..2] = lambda Ex, Ey, Hz; [3..6] = lambda psi_hz_x,
// psi_hz_y, psi_ex_y, psi_ey_x.
template <typename T>
struct TBAdjArgs {
  SimArgs<T> s;  // geometry, coefficients and strips (its field pointers are not used)
  const T* in[7];
  T* out[7];
  const T* trace;       // Hz^(n+1/2) on [ti0, ti0+tnx) x [tj0, tj0+tny) per step, from ctl[1]
  const int64_t* ctl;   // device: ctl[0] = top step of the current launch block, ctl[1] = trace_n0
  int ti0, tnx, tj0, tny;
  int i0, nxd, j0, nyd;  // design cells
  double *gx, *gy;       // dJ/dcb_ex (nxd, nyd+1), dJ/dcb_ey (nxd+1, nyd)
  T* ltrace;             // lambda Ex, Ey of the window box (nxd+1, nyd+1) per step of the block:
                         // [ctl[0] - 1 - n][component][i - i0][j - j0]
  int n_hsrc, n_esrc;
  AdjSrc<T> hsrc[MAX_SRC_NODES], esrc[MAX_SRC_NODES];
};

// Tile shape of the adjoint kernels of a dtype (rows ER, columns EC, depth K).
void tb_adj_shape(int dtype, int* ER, int* EC, int* K);

template <typename T>
int tb_adj_attrs();

// Reverse steps n_hi-1 … n_hi-K of one simulation, n_hi = ctl[0] - step_off: interior tiles
// (tiles[0, n_inner)) on `main`, then n_kind[0..2] CPML tiles of kinds X, Y, XY, each kind on
// its side stream (fork/join through the events). Capturable in a CUDA graph: the step comes
// from device memory.
template <typename T>
int tb_adj_launch(const TBAdjArgs<T>& a, const int2* tiles, int n_inner, const int* n_kind, int step_off,
                  cudaStream_t main, const cudaStream_t* sides, cudaEvent_t fork, const cudaEvent_t* joins);

// The same for a batch: args is a device array of 2 TBAdjArgs per simulation (reading the
// primary or the second buffer), tiles (sim, r0, c0, kind): interior tiles, then the CPML
// tiles sorted by kind.
template <typename T>
int tb_adj_batch_launch(const TBAdjArgs<T>* args, const int4* tiles, int n_inner, const int* n_kind, int parity,
                        int step_off, cudaStream_t main, const cudaStream_t* sides, cudaEvent_t fork,
                        const cudaEvent_t* joins);

// ctl[0] += delta (one thread), for the end of a captured block of launches.
void tb_adj_ctl_add(int64_t* ctl, int64_t delta, cudaStream_t s);

// dJ/dcb += the recorded steps ctl[0]-1 … ctl[0]-n_slots of n_designs designs (device args,
// args[stride * k]); max_nodes = the largest nxd*(nyd+1) + (nxd+1)*nyd.
template <typename T>
void tb_adj_grad(const TBAdjArgs<T>* args, int stride, int n_designs, int64_t max_nodes, int n_slots, cudaStream_t s);

}  // namespace etg
