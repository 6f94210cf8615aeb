// Temporally blocked kernel family of the resident simulation (several steps per launch).
#pragma once

#include <vector>

#include "etg_sim.h"

namespace etg {

struct TBState;

TBState* tb_create();
void tb_destroy(TBState* tb);
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
void tb_default_shape(int dtype, int* ER, int* EC, int* K);

// Tiles of the default shape over a grid: interior tiles first, then CPML tiles.
void tb_tiles(int dtype, int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi,
              std::vector<int2>* tiles, int* n_inner);

// One launch pair (interior, then CPML tiles) of the default shape, src -> dst, on one stream,
// for callers that hold both buffers and the tile list themselves.
template <typename T>
cudaError_t tb_default_launch(const SimArgs<T>& src, const SimArgs<T>& dst, const int2* tiles,
                              int n_inner, int n_pml, int step_off, cudaStream_t s);

}  // namespace etg
