// Temporally blocked kernel family of the resident simulation (several steps per launch).
#pragma once

#include <vector>

#include "etg_sim.h"

namespace etg {

struct TBState;

// Destination planes of one temporally blocked launch.
template <typename T>
struct TBDst {
  T *ex, *ey, *hz, *psi_ex_y, *psi_ey_x, *psi_hz_x, *psi_hz_y;
};

// One simulation of a batch: its arguments with the fields of either buffer as the source.
template <typename T>
struct BatchSim {
  SimArgs<T> src[2];  // [0]: read A (the simulation's fields), [1]: read B (the second buffer)
  TBDst<T> dst[2];    // [0]: write B, [1]: write A
  PhasePlan<T> ph, pe;
};

// Batched launch pair (interior tiles without a plan on `main`; the CPML tiles of each kind
// and the interior tiles with a source, monitor or trace node each on a side stream, sides[0..3])
// of the compiled shape with ER rows, depth K and NW warps; `sims` is a device array of
// BatchSim<T>, `tiles` (sim, r0, c0, kind): interior tiles first (the n_hot with a plan
// leading), then n_kind[0..2] tiles of kinds X, Y, XY, of which the leading n_kind[3..5] have
// a source, monitor or trace node (they run with the plan code on sides[3]).
template <typename T>
int tb_batch_pair(int ER, int K, int NW, const void* sims, const int4* tiles, int n_inner, int n_hot,
                  const int* n_kind, int parity, int step_off, cudaStream_t main, const cudaStream_t* sides,
                  cudaEvent_t fork, const cudaEvent_t* joins);
template <typename T>
int tb_batch_attrs(int ER, int K, int NW);
// Block DFT of a batch: every simulation's sampled monitors (at most max_mon per simulation,
// at most max_work frequencies x nodes each) summed over the block's n_slots steps.
template <typename T>
void tb_batch_dft(const void* sims, int n_sims, int64_t max_work, int max_mon, int n_slots, cudaStream_t s);
// Output tiles of one grid, interior tiles first; tiles meeting a `hot` rectangle lead each kind.
// A CPML tile carries its kind (1: CPML across rows, 2: across columns, 3: both) in bits
// 28-29 of .x (tb_tile_row and tb_tile_kind take it apart).
// Adds to `into` the rectangles of `add` it lacks (restarting from `add` past `cap`); true if
// any was new. Tile lists split on such a union keep a tile's kernel across runs with and
// without monitors or traces.
bool tb_hot_union(std::vector<int4>* into, const std::vector<int4>& add, size_t cap);
// *n_hot (if given): the leading interior tiles that meet a `hot` rectangle.
// *kind_hot (if given, three counts): the leading CPML tiles of each kind that meet one.
void tb_split_tiles(int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi, int ER, int EC, int K,
                    const std::vector<int4>& hot, std::vector<int2>* tiles, int* n_inner, int* n_hot = nullptr,
                    int* kind_hot = nullptr);

inline int tb_tile_row(int2 t) { return t.x & ((1 << 28) - 1); }
// Column segments (k_tb_seg) of the current tile list, 0 if it uses none.
int tb_segments(const TBState* tb);
inline int tb_tile_kind(int2 t) { return t.x >> 28; }

TBState* tb_create();
void tb_destroy(TBState* tb);
// Kernel time (ms), launches and output cells per launch of the last advance run with
// ETG_OPT_TIMING 2, for [interior tiles without a plan (the lean kernel), every other tile
// (CPML and interior tiles with sources, monitors or traces), CPML X tiles alone, Y alone,
// XY alone] (zeros
// otherwise or before any temporally blocked advance).
void tb_kernel_timing(const TBState* tb, double* ms, int64_t* launches, int64_t* cells);
void tb_invalidate(TBState* tb);  // drop cached graphs and plans (pointers changed)

// Whether the temporally blocked path handles a grid of this size.
template <typename T>
bool tb_supported(int nx, int ny);

// Advance n_steps from the step counter in a.step, leaving the result in the fields of `a`.
template <typename T>
int tb_advance(TBState* tb, const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
               int64_t n_steps, const int64_t* opt, cudaStream_t s);

}  // namespace etg

namespace etg {

// Default tile shape of the temporally blocked kernel for a dtype: rows, columns, depth K.
void tb_default_shape(int dtype, int* ER, int* EC, int* K, int kernel = 0);  // kernel 3: the TMA kernel's

// Tiles of the default shape over a grid: interior tiles first, then CPML tiles.
void tb_tiles(int dtype, int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi,
              std::vector<int2>* tiles, int* n_inner);

// One launch pair (interior, then CPML tiles) of the default shape, src -> dst, on one stream,
// for callers that hold both buffers and the tile list themselves.
template <typename T>
cudaError_t tb_default_launch(const SimArgs<T>& src, const SimArgs<T>& dst, const int2* tiles,
                              int n_inner, int n_pml, int step_off, cudaStream_t s);

}  // namespace etg
