// Temporally blocked kernel family of the resident simulation (several steps per launch).
#pragma once

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
