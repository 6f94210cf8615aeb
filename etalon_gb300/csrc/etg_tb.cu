// Temporally blocked kernels: not enabled yet; the one-step kernels run every advance.
#include "etg_tb.h"

namespace etg {

struct TBState {};

TBState* tb_create() { return new TBState; }
void tb_destroy(TBState* tb) { delete tb; }
void tb_invalidate(TBState*) {}

template <typename T>
bool tb_supported(int, int) { return false; }

template <typename T>
int tb_advance(TBState*, const SimArgs<T>&, const PhasePlan<T>&, const PhasePlan<T>&, int64_t,
               const int64_t*, cudaStream_t) {
  set_error("temporally blocked kernel not available in this build");
  return ETG_ERR_STATE;
}

template bool tb_supported<float>(int, int);
template bool tb_supported<double>(int, int);
template int tb_advance<float>(TBState*, const SimArgs<float>&, const PhasePlan<float>&,
                               const PhasePlan<float>&, int64_t, const int64_t*, cudaStream_t);
template int tb_advance<double>(TBState*, const SimArgs<double>&, const PhasePlan<double>&,
                                const PhasePlan<double>&, int64_t, const int64_t*, cudaStream_t);

}  // namespace etg
