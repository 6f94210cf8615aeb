// Batched launches of the temporally blocked kernels: the tiles of many grids in one launch
// per kind (the tile body and kernels are in etg_tb_tile.cuh).
#include <vector>

#include "etg_tb.h"
#include "etg_tb_tile.cuh"

namespace etg {

// ------------------------------------------------------------------------ batched launches

// One kind's CPML tiles of a batch: the leading n_hot with the plan code on `hot`, the rest lean on `s`.
template <typename T, int RP, int K, int KIND>
static cudaError_t batch_kind(const BatchSim<T>* b, const int4* tiles, int n, int n_hot, int parity, int step_off,
                              cudaStream_t s, cudaStream_t hot) {
  constexpr size_t SMEM = TBShape<T, RP, K, KIND>::SMEM;
  if (n_hot) {
    k_tb_batch_kind<T, RP, K, KIND, 8, true><<<n_hot, dim3(32, 8), SMEM, hot>>>(b, tiles, parity, step_off);
    g_launches += 1;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (n > n_hot) {
    k_tb_batch_kind<T, RP, K, KIND, 8, false><<<n - n_hot, dim3(32, 8), SMEM, s>>>(b, tiles + n_hot, parity,
                                                                                   step_off);
    g_launches += 1;
    return cudaGetLastError();
  }
  return cudaSuccess;
}

template <typename T, int RPT, int K, int NW>
static cudaError_t batch_pair(const void* sims, const int4* tiles, int n_inner, int n_hot, const int* n_kind,
                              int parity, int step_off, cudaStream_t main, const cudaStream_t* sides,
                              cudaEvent_t fork, const cudaEvent_t* joins) {
  constexpr int RP = RPT * NW / 8;  // CPML tiles: 8 warps over the same rows, one kernel per kind
  const BatchSim<T>* b = (const BatchSim<T>*)sims;
  cudaError_t e = cudaEventRecord(fork, main);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(sides[k], fork, 0);
  const int4* t = tiles + n_inner;
  if (e == cudaSuccess) e = batch_kind<T, RP, K, KIND_X>(b, t, n_kind[0], n_kind[3], parity, step_off, sides[0], sides[3]);
  t += n_kind[0];
  if (e == cudaSuccess) e = batch_kind<T, RP, K, KIND_Y>(b, t, n_kind[1], n_kind[4], parity, step_off, sides[1], sides[3]);
  t += n_kind[1];
  if (e == cudaSuccess)
    e = batch_kind<T, RP, K, KIND_XY>(b, t, n_kind[2], n_kind[5], parity, step_off, sides[2], sides[3]);
  if (e == cudaSuccess && n_hot) {
    k_tb_batch<T, RPT, K, false, NW, true><<<n_hot, dim3(32, NW), tb_smem<T, RPT, K, false, NW>(), sides[3]>>>(
        b, tiles, parity, step_off);
    g_launches += 1;
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && n_inner > n_hot) {
    k_tb_batch<T, RPT, K, false, NW, false><<<n_inner - n_hot, dim3(32, NW), tb_smem<T, RPT, K, false, NW>(), main>>>(
        b, tiles + n_hot, parity, step_off);
    g_launches += 1;
    e = cudaGetLastError();
  }
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
    e = cudaEventRecord(joins[k], sides[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(main, joins[k], 0);
  }
  return e;
}

template <typename T, int RPT, int K, int NW>
static cudaError_t batch_attrs() {
  constexpr int RP = RPT * NW / 8;
  cudaError_t e = cudaFuncSetAttribute(k_tb_batch<T, RPT, K, false, NW, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tb_smem<T, RPT, K, false, NW>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tb_batch<T, RPT, K, false, NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tb_smem<T, RPT, K, false, NW>());
#define ETG_BATCH_KIND_ATTR(KD, PL)                                                                   \
  if (e == cudaSuccess)                                                                              \
    e = cudaFuncSetAttribute(k_tb_batch_kind<T, RP, K, KD, 8, PL>,                                   \
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TBShape<T, RP, K, KD>::SMEM);
  ETG_BATCH_KIND_ATTR(KIND_X, true)
  ETG_BATCH_KIND_ATTR(KIND_X, false)
  ETG_BATCH_KIND_ATTR(KIND_Y, true)
  ETG_BATCH_KIND_ATTR(KIND_Y, false)
  ETG_BATCH_KIND_ATTR(KIND_XY, true)
  ETG_BATCH_KIND_ATTR(KIND_XY, false)
#undef ETG_BATCH_KIND_ATTR
  return e;
}

template <typename T>
int tb_batch_pair(int ER, int K, int NW, const void* sims, const int4* tiles, int n_inner, int n_hot,
                  const int* n_kind, int parity, int step_off, cudaStream_t main, const cudaStream_t* sides,
                  cudaEvent_t fork, const cudaEvent_t* joins) {
#define ETG_BATCH_CASE(DT, R, KK, NWW)                                                                        \
  if ((int)sizeof(T) == DT && ER == NWW * R && K == KK && NW == NWW) {                                        \
    ETG_TRY_CUDA((batch_pair<T, R, KK, NWW>(sims, tiles, n_inner, n_hot, n_kind, parity, step_off, main, sides, \
                                            fork, joins)));                                                    \
    return ETG_OK;                                                                                            \
  }
  if constexpr (sizeof(T) == 4) {
    ETG_TB_SHAPES_F32(ETG_BATCH_CASE)
  } else {
    ETG_TB_SHAPES_F64(ETG_BATCH_CASE)
  }
#undef ETG_BATCH_CASE
  set_error("no compiled batched kernel with %d rows, depth %d and %d warps", ER, K, NW);
  return ETG_ERR_ARGUMENT;
}

template <typename T>
int tb_batch_attrs(int ER, int K, int NW) {
#define ETG_BATCH_ATTR(DT, R, KK, NWW)                             \
  if ((int)sizeof(T) == DT && ER == NWW * R && K == KK && NW == NWW) { \
    ETG_TRY_CUDA((batch_attrs<T, R, KK, NWW>()));                  \
    return ETG_OK;                                                 \
  }
  if constexpr (sizeof(T) == 4) {
    ETG_TB_SHAPES_F32(ETG_BATCH_ATTR)
  } else {
    ETG_TB_SHAPES_F64(ETG_BATCH_ATTR)
  }
#undef ETG_BATCH_ATTR
  set_error("no compiled batched kernel with %d rows, depth %d and %d warps", ER, K, NW);
  return ETG_ERR_ARGUMENT;
}

template int tb_batch_pair<float>(int, int, int, const void*, const int4*, int, int, const int*, int, int,
                                  cudaStream_t, const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);
template int tb_batch_pair<double>(int, int, int, const void*, const int4*, int, int, const int*, int, int,
                                   cudaStream_t, const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);
template int tb_batch_attrs<float>(int, int, int);
template int tb_batch_attrs<double>(int, int, int);

}  // namespace etg
