// Temporally blocked 2D TE kernels: K whole time steps per launch, one HBM pass.
//
// The grid of cells (i, j) in [0, nx] x [0, ny] — each cell holding Hz(i, j), Ex(i, j),
// Ey(i, j) on the shared pitched index i * P + j — is cut into output tiles of OR x OC
// cells. A CTA loads its tile plus a halo of K cells on every side (one leapfrog step reads
// at most one neighbour in each direction, so K steps need K cells), advances the extended
// tile K steps on chip, and writes the output tile to the other buffer of a ping-pong pair.
// Halo cells are recomputed by every tile that needs them, from the same inputs with the
// same operations, so they are bit-identical to the owner's values; point sources are
// injected wherever a tile holds the node, and DFT monitors accumulate only in the owning
// tile, in step order. After step s only cells at least s from the tile edge are valid; the
// edge cells see zeros beyond the tile and are never used for an output cell.
//
// Mapping: warp ty owns the RPT consecutive rows [ty*RPT, (ty+1)*RPT) of the extended tile
// (ER = 8 RPT rows), lane l the W columns [W l, W l + W) (EC = 32 W, one 16-byte access per
// row). Each thread keeps Ex, Ey, Hz of its RPT x W cells in registers for all K steps:
// column neighbours come from the adjacent lane by shuffle, row neighbours from its own
// registers, and only a warp's first row of Ey and last row of Hz cross to the warps above
// and below, through shared memory, behind the two barriers of each step. cb (and psi in
// CPML tiles) sit in shared memory, read only by the owning thread.
//
// Interior tiles — extended region inside [1, nx) x [1, ny) and inside the unit rectangle,
// where c = 0 and 1/kappa = 1 exactly — take the lean update: Etalon's CPML terms are
// b*0 + 0*d = +0 and d * 1 = d there, so its expression reduces exactly to "d + 0" for finite
// d, and no cell of such a tile is a PEC edge. CPML tiles run Etalon's full expression with
// per-cell domain checks.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "etg_tb.h"
#include "etg_tb_tile.cuh"

namespace etg {

// ------------------------------------------------------------------------ persistent TMA variant
//
// Two CTAs per SM walk the tile list (interior tiles first, then CPML tiles) with stride
// gridDim.x. Ex, Ey, Hz, cb_ex and cb_ey of an extended tile arrive by TMA
// (cp.async.bulk.tensor.2d, zero fill outside the arrays) into the CTA's stage, completion
// tracked by an mbarrier. The threads copy their cells (fields and cb) to registers at once,
// so the stage is free again: the next tile's TMA runs while this tile takes its K steps,
// and the two CTAs of an SM hide each other's barriers. A CPML tile instead fills the stage
// with its four psi planes and its CPML profiles and fetches the next tile after it.
// The arithmetic, injection, DFT and trace are those of k_tb_step.

struct TMAMaps {
  CUtensorMap ex, ey, hz, cbx, cby;
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_load_tile(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Iteration limit of the first attempt of every bounded stage wait. Tests lower it (see
// etg_debug_set_wait_tries) to make the wait give up on a real, completing copy.
constexpr uint32_t kWaitTries = 1u << 20;
__device__ uint32_t g_wait_tries = kWaitTries;

// Wait for the stage with an iteration limit; on time-out flag the error, wait once more
// (bounded) for the copy still in flight, and report failure so the CTA can return.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* flag) {
  const uint32_t tries = *(volatile uint32_t*)&g_wait_tries;
  for (uint32_t it = 0; it < tries; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 32) __nanosleep(128);
  }
  atomicOr(flag, ERRBIT_TIMEOUT);
  for (uint32_t it = 0; it < (1u << 20); ++it) {
    if (mbar_try_wait(bar, parity)) break;
    __nanosleep(128);
  }
  return false;
}

template <typename T, int RPT, int K>
struct TMAShape {
  static constexpr int W = TBVec<T>::W;
  static constexpr int ER = 8 * RPT, EC = 32 * W, OR = ER - 2 * K, OC = EC - 2 * K;
  static constexpr int PL = ER * EC;
  static constexpr int STAGE = 5 * PL;       // Ex, Ey, Hz, cb_ex, cb_ey; a CPML tile's psi after the copy
  static constexpr int PROF = 6 * (ER + EC);  // CPML profiles of a tile: 6 per row, 6 per column
  static constexpr int XCH = 9 * EC;
  static constexpr uint32_t TX_BYTES = (uint32_t)(5 * PL * sizeof(T));
  static constexpr size_t SMEM = (size_t)(STAGE + PROF + 2 * XCH) * sizeof(T) + sizeof(uint64_t) + 128;
  static_assert(K % W == 0 && OR > 0 && OC > 0, "tile shape");
  static_assert((PL * sizeof(T)) % 128 == 0, "stage planes stay 128-byte aligned");
};

template <typename T, int RPT, int K>
__global__ void __launch_bounds__(TB_THREADS, 2)
k_tb_tma(const __grid_constant__ TMAMaps maps, const __grid_constant__ SimArgs<T> a,
         const __grid_constant__ TBDst<T> dst, const int2* __restrict__ tiles, int n_inner, int n_tiles,
         const __grid_constant__ PhasePlan<T> ph, const __grid_constant__ PhasePlan<T> pe, int step_off) {
  using S = TMAShape<T, RPT, K>;
  using Vw = TBVec<T>;
  constexpr int W = S::W, ER = S::ER, EC = S::EC, PL = S::PL;
  extern __shared__ __align__(128) unsigned char tma_smem[];
  // TMA destination on a 128-byte boundary whatever the base of dynamic shared memory
  T* const stage = reinterpret_cast<T*>(tma_smem + ((128u - (smem_addr(tma_smem) & 127u)) & 127u));
  T* const prof = stage + S::STAGE;  // bxh cxh kxh bxe cxe kxe [ER each], byh cyh kyh bye cye kye [EC each]
  T* const sHzX = prof + S::PROF;
  T* const sEyX = sHzX + S::XCH;
  uint64_t* const mbar = reinterpret_cast<uint64_t*>(sEyX + S::XCH);
  __shared__ uint32_t s_rel[4];

  const int lane = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + lane;
  const int nx = a.nx, ny = a.ny;
  const int64_t P = a.P;
  const int lj0 = W * lane, lr0 = RPT * ty;
  if ((int)blockIdx.x >= n_tiles) return;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (ty == 0) {
    Vw z;
    z.zero();
    z.st(sHzX + lj0);  // the row above every tile
  }
  if (ty == 7) {
    Vw z;
    z.zero();
    z.st(sEyX + 8 * EC + lj0);  // the row below every tile
  }
  __syncthreads();
  auto fetch = [&](int k) {  // one thread
    const int2 t = make_int2(tiles[k].x & ((1 << KIND_SHIFT) - 1), tiles[k].y);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(S::TX_BYTES)
                 : "memory");
    const int x = t.y - K, y = t.x - K;
    tma_load_tile(stage + 0 * PL, &maps.ex, x, y, mbar);
    tma_load_tile(stage + 1 * PL, &maps.ey, x, y, mbar);
    tma_load_tile(stage + 2 * PL, &maps.hz, x, y, mbar);
    tma_load_tile(stage + 3 * PL, &maps.cbx, x, y, mbar);
    tma_load_tile(stage + 4 * PL, &maps.cby, x, y, mbar);
  };
  if (tid == 0) fetch(blockIdx.x);
  uint32_t parity = 0;
  const T db = a.db, idx = a.inv_dx, idy = a.inv_dy;
  const int64_t n_base = *a.step + step_off;

  for (int k = blockIdx.x; k < n_tiles; k += gridDim.x) {
    const int2 tile = make_int2(tiles[k].x & ((1 << KIND_SHIFT) - 1), tiles[k].y);
    const bool pml = k >= n_inner;
    const int next = k + gridDim.x;
    const int R0 = tile.x - K, C0 = tile.y - K, j0 = C0 + lj0, i0 = R0 + lr0;
    const bool lane_in = j0 >= 0 && j0 + W <= P;
    T* const sPsi = stage;  // CPML tiles: psi_hz_x, psi_hz_y, psi_ex_y, psi_ey_x after the copy
    if (ty == 0) {
      auto src_hits = [&](const PhasePlan<T>& p) {
        bool hit = false;
        if (lane < p.n_src) {
          const SrcDesc<T>& d = p.src[lane];
          hit = d.i >= R0 && d.i < R0 + ER && d.j >= C0 && d.j < C0 + EC;
        }
        return __ballot_sync(0xffffffffu, hit);
      };
      auto mon_hits = [&](const PhasePlan<T>& p) {
        bool hit = false;
        if (lane < p.n_mon) {
          const MonDesc<T>& d = p.mon[lane];
          hit = d.ix0 < tile.x + S::OR && d.ix0 + d.nxm > tile.x && d.jy0 < tile.y + S::OC && d.jy0 + d.nym > tile.y;
        }
        return __ballot_sync(0xffffffffu, hit);
      };
      const uint32_t r0 = src_hits(ph), r1 = src_hits(pe), r2 = mon_hits(ph), r3 = mon_hits(pe);
      if (lane == 0) {
        s_rel[0] = r0;
        s_rel[1] = r1;
        s_rel[2] = r2;
        s_rel[3] = r3;
      }
    }
    const bool landed = mbar_wait_bounded(mbar, parity, a.flag);
    parity ^= 1;
    // leave together: a thread that gave up has also waited (bounded) for the copy in flight
    if (!__syncthreads_and(landed)) return;
    Vw ex[RPT], ey[RPT], hz[RPT], cbx[RPT], cby[RPT];
#pragma unroll
    for (int t = 0; t < RPT; ++t) {
      const int o = (lr0 + t) * EC + lj0;
      ex[t].ld(stage + 0 * PL + o);
      ey[t].ld(stage + 1 * PL + o);
      hz[t].ld(stage + 2 * PL + o);
      cbx[t].ld(stage + 3 * PL + o);
      cby[t].ld(stage + 4 * PL + o);
    }
    ey[0].st(sEyX + ty * EC + lj0);
    __syncthreads();  // the stage is copied out
    if (!pml && next < n_tiles && tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      fetch(next);
    }
    if (pml) {  // psi planes into the stage, CPML profiles of the tile's rows and columns
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = i0 + t;
        const bool in = lane_in && (unsigned)i <= (unsigned)nx;
        const int64_t g = (int64_t)i * P + j0;
        const int o = (lr0 + t) * EC + lj0;
        Vw p0, p1, p2, p3;
        if (in) {
          p0.ld(a.psi_hz_x + g);
          p1.ld(a.psi_hz_y + g);
          p2.ld(a.psi_ex_y + g);
          p3.ld(a.psi_ey_x + g);
        } else {
          p0.zero();
          p1.zero();
          p2.zero();
          p3.zero();
        }
        p0.st(sPsi + 0 * PL + o);
        p1.st(sPsi + 1 * PL + o);
        p2.st(sPsi + 2 * PL + o);
        p3.st(sPsi + 3 * PL + o);
      }
      for (int r = tid; r < ER; r += TB_THREADS) {
        const int i = R0 + r, ih = min(max(i, 0), nx - 1), ie = min(max(i, 0), nx);
        prof[0 * ER + r] = a.bx_h[ih];
        prof[1 * ER + r] = a.cx_h[ih];
        prof[2 * ER + r] = a.ikx_h[ih];
        prof[3 * ER + r] = a.bx_e[ie];
        prof[4 * ER + r] = a.cx_e[ie];
        prof[5 * ER + r] = a.ikx_e[ie];
      }
      for (int c = tid; c < EC; c += TB_THREADS) {
        const int j = C0 + c, jh = min(max(j, 0), ny - 1), je = min(max(j, 0), ny);
        T* py = prof + 6 * ER;
        py[0 * EC + c] = a.by_h[jh];
        py[1 * EC + c] = a.cy_h[jh];
        py[2 * EC + c] = a.iky_h[jh];
        py[3 * EC + c] = a.by_e[je];
        py[4 * EC + c] = a.cy_e[je];
        py[5 * EC + c] = a.iky_e[je];
      }
      __syncthreads();
    }
    const T* const px = prof;           // per tile row
    const T* const pyc = prof + 6 * ER;  // per tile column
    const uint32_t relSrcH = s_rel[0], relSrcE = s_rel[1], relMonH = s_rel[2], relMonE = s_rel[3];
    const int t_lo = max(0, K - lr0), t_hi = min(RPT, ER - K - lr0);
    const int e_lo = lj0 >= K ? 0 : W, e_hi = lj0 + W <= EC - K ? W : 0;
    const bool traced = ph.trace.buf && ph.trace.ti0 < tile.x + S::OR && ph.trace.ti0 + ph.trace.tnx > tile.x &&
                        ph.trace.tj0 < tile.y + S::OC && ph.trace.tj0 + ph.trace.tny > tile.y;

    for (int s = 0; s < K; ++s) {
      const int64_t n = n_base + s;
      {  // H half step
        Vw eyb;
        eyb.ld(sEyX + (ty + 1) * EC + lj0);
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          T exr = __shfl_down_sync(0xffffffffu, ex[t].v[0], 1);
          if (lane == 31) exr = zero<T>();
#pragma unroll
          for (int e = 0; e < W; ++e) {
            const T exn = e < W - 1 ? ex[t].v[e + 1] : exr;
            const T eyn = t < RPT - 1 ? ey[t + 1].v[e] : eyb.v[e];
            const T dex_dy = mul(sub(exn, ex[t].v[e]), idy);
            const T dey_dx = mul(sub(eyn, ey[t].v[e]), idx);
            if (!pml) {
              hz[t].v[e] = add(hz[t].v[e], mul(db, sub(add(dex_dy, zero<T>()), add(dey_dx, zero<T>()))));
            } else {
              const int i = i0 + t, j = j0 + e, r = lr0 + t, c = lj0 + e;
              if (i >= 0 && i < nx && j >= 0 && j < ny) {
                T* pxp = sPsi + 0 * PL + r * EC + c;
                T* pyp = sPsi + 1 * PL + r * EC + c;
                const T py = add(mul(pyc[0 * EC + c], *pyp), mul(pyc[1 * EC + c], dex_dy));
                const T pxv = add(mul(px[0 * ER + r], *pxp), mul(px[1 * ER + r], dey_dx));
                if (j < a.ys_lo || j >= a.ys_hi) *pyp = py;
                if (i < a.xs_lo || i >= a.xs_hi) *pxp = pxv;
                hz[t].v[e] = add(hz[t].v[e], mul(db, sub(add(mul(dex_dy, pyc[2 * EC + c]), py),
                                                         add(mul(dey_dx, px[2 * ER + r]), pxv))));
              }
            }
          }
        }
      }
      if (relSrcH) tb_inject<T, RPT, W>(ph, relSrcH, ex, ey, hz, i0, j0, n, a.flag);
      if (relMonH) {
        for (uint32_t m = relMonH; m; m &= m - 1) {
          const MonDesc<T>& d = ph.mon[__ffs(m) - 1];
          const int64_t r = n - d.n0;
          if (r < 0 || r >= d.rows) atomicOr(a.flag, ERRBIT_TABLE);
          else tb_dft<T, RPT, W>(d, hz, i0, j0, t_lo, t_hi, e_lo, e_hi, r);
        }
      }
      if (traced) {
        const TraceDesc<T>& tr = ph.trace;
        const int64_t r = n - tr.n0;
        if (r < 0 || r >= tr.rows) {
          atomicOr(a.flag, ERRBIT_TABLE);
        } else {
#pragma unroll
          for (int t = 0; t < RPT; ++t) {
            const unsigned di = (unsigned)(i0 + t - tr.ti0);
            if (t < t_lo || t >= t_hi || di >= (unsigned)tr.tnx) continue;
#pragma unroll
            for (int e = 0; e < W; ++e) {
              const unsigned dj = (unsigned)(j0 + e - tr.tj0);
              if (e >= e_lo && e < e_hi && dj < (unsigned)tr.tny) tr.buf[(r * tr.tnx + di) * tr.tny + dj] = hz[t].v[e];
            }
          }
        }
      }
      hz[RPT - 1].st(sHzX + (ty + 1) * EC + lj0);
      __syncthreads();
      {  // E half step
        Vw hza;
        hza.ld(sHzX + ty * EC + lj0);
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          T hzl = __shfl_up_sync(0xffffffffu, hz[t].v[W - 1], 1);
          if (lane == 0) hzl = zero<T>();
#pragma unroll
          for (int e = 0; e < W; ++e) {
            const T hzp = e > 0 ? hz[t].v[e - 1] : hzl;
            const T hzu = t > 0 ? hz[t - 1].v[e] : hza.v[e];
            const T dy = mul(sub(hz[t].v[e], hzp), idy);
            const T dx = mul(sub(hz[t].v[e], hzu), idx);
            if (!pml) {
              ex[t].v[e] = add(ex[t].v[e], mul(cbx[t].v[e], add(dy, zero<T>())));
              ey[t].v[e] = sub(ey[t].v[e], mul(cby[t].v[e], add(dx, zero<T>())));
            } else {
              const int i = i0 + t, j = j0 + e, r = lr0 + t, c = lj0 + e;
              if (i >= 0 && i < nx && j >= 1 && j <= ny - 1) {
                T* pp = sPsi + 2 * PL + r * EC + c;
                const T p = add(mul(pyc[3 * EC + c], *pp), mul(pyc[4 * EC + c], dy));
                if (j < a.ys_lo || j >= a.ys_hi) *pp = p;
                ex[t].v[e] = add(ex[t].v[e], mul(cbx[t].v[e], add(mul(dy, pyc[5 * EC + c]), p)));
              }
              if (i >= 1 && i <= nx - 1 && j >= 0 && j < ny) {
                T* pp = sPsi + 3 * PL + r * EC + c;
                const T p = add(mul(px[3 * ER + r], *pp), mul(px[4 * ER + r], dx));
                if (i < a.xs_lo || i >= a.xs_hi) *pp = p;
                ey[t].v[e] = sub(ey[t].v[e], mul(cby[t].v[e], add(mul(dx, px[5 * ER + r]), p)));
              }
            }
          }
        }
      }
      if (relSrcE) tb_inject<T, RPT, W>(pe, relSrcE, ex, ey, hz, i0, j0, n, a.flag);
      if (relMonE) {
        for (uint32_t m = relMonE; m; m &= m - 1) {
          const MonDesc<T>& d = pe.mon[__ffs(m) - 1];
          const int64_t r = n - d.n0;
          if (r < 0 || r >= d.rows) atomicOr(a.flag, ERRBIT_TABLE);
          else if (d.comp == ETG_EX) tb_dft<T, RPT, W>(d, ex, i0, j0, t_lo, t_hi, e_lo, e_hi, r);
          else tb_dft<T, RPT, W>(d, ey, i0, j0, t_lo, t_hi, e_lo, e_hi, r);
        }
      }
      ey[0].st(sEyX + ty * EC + lj0);
      __syncthreads();
    }

    // write the output tile
    if (e_lo == 0 && e_hi == W && lane_in) {
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int i = i0 + t;
        if (t < t_lo || t >= t_hi || (unsigned)i > (unsigned)nx) continue;
        const int64_t g = (int64_t)i * P + j0;
        ex[t].st(dst.ex + g);
        ey[t].st(dst.ey + g);
        hz[t].st(dst.hz + g);
        if (pml) {
          const int o = (lr0 + t) * EC + lj0;
          Vw v;
          v.ld(sPsi + 0 * PL + o);
          v.st(dst.psi_hz_x + g);
          v.ld(sPsi + 1 * PL + o);
          v.st(dst.psi_hz_y + g);
          v.ld(sPsi + 2 * PL + o);
          v.st(dst.psi_ex_y + g);
          v.ld(sPsi + 3 * PL + o);
          v.st(dst.psi_ey_x + g);
        }
      }
    }
    if (pml) {
      __syncthreads();  // every thread is done with the psi planes in the stage
      if (next < n_tiles && tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fetch(next);
      }
    }
  }
}

// ------------------------------------------------------------------------ block DFT
//
// Tiles that hold monitor nodes record them per step (tb_sample); after each block of
// launches one thread per (monitor, frequency, node) adds the block's samples to its
// accumulator in step order. Done in the tile itself, those serial read-modify-writes made
// the monitor tiles the longest of every launch.

template <typename T>
__global__ void k_dft_block(const __grid_constant__ PhasePlan<T> ph, const __grid_constant__ PhasePlan<T> pe,
                            const int64_t* __restrict__ step, int n_slots, int* flag) {
  const int m = blockIdx.y;
  const MonDesc<T>& d = m < ph.n_mon ? ph.mon[m] : pe.mon[m - ph.n_mon];
  dft_block_node(d, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, *step, n_slots, flag);
}

template <typename T>
__global__ void k_dft_block_batch(const BatchSim<T>* __restrict__ sims, int n_slots) {
  const BatchSim<T>& b = sims[blockIdx.y];
  const int m = blockIdx.z;
  if (m >= b.ph.n_mon + b.pe.n_mon) return;
  const MonDesc<T>& d = m < b.ph.n_mon ? b.ph.mon[m] : b.pe.mon[m - b.ph.n_mon];
  dft_block_node(d, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, *b.src[0].step, n_slots, b.src[0].flag);
}

// Largest (frequencies x nodes) of the sampled monitors of a plan pair; 0 when none samples.
template <typename T>
static int64_t sampled_work(const PhasePlan<T>& ph, const PhasePlan<T>& pe, int* n_mon) {
  int64_t w = 0;
  *n_mon = ph.n_mon + pe.n_mon;
  for (int m = 0; m < *n_mon; ++m) {
    const MonDesc<T>& d = m < ph.n_mon ? ph.mon[m] : pe.mon[m - ph.n_mon];
    if (d.samp) w = std::max<int64_t>(w, (int64_t)d.nxm * d.nym * d.n_f);
  }
  return w;
}

template <typename T>
void launch_dft_block(const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe, int n_slots,
                      cudaStream_t s) {
  int n_mon = 0;
  const int64_t w = sampled_work(ph, pe, &n_mon);
  if (w == 0 || n_slots == 0) return;
  k_dft_block<T><<<dim3((unsigned)((w + 127) / 128), (unsigned)n_mon), 128, 0, s>>>(ph, pe, a.step, n_slots, a.flag);
  g_launches += 1;
}

template <typename T>
void tb_batch_dft(const void* sims, int n_sims, int64_t max_work, int max_mon, int n_slots, cudaStream_t s) {
  if (max_work == 0 || n_slots == 0) return;
  const dim3 grid((unsigned)((max_work + 127) / 128), (unsigned)n_sims, (unsigned)max_mon);
  k_dft_block_batch<T><<<grid, 128, 0, s>>>((const BatchSim<T>*)sims, n_slots);
  g_launches += 1;
}

template void tb_batch_dft<float>(const void*, int, int64_t, int, int, cudaStream_t);
template void tb_batch_dft<double>(const void*, int, int64_t, int, int, cudaStream_t);

// ------------------------------------------------------------------------ persistent pipelined kernel
//
// One CTA per SM claims tiles from a device counter until none is left: CPML tiles first
// (the long ones, each loading itself), then interior tiles. While an interior tile runs its
// K steps, TMA brings the next interior tile's Ex, Ey, Hz into the stage and its cb into the
// other cb buffer, so the load of every interior tile but a CTA's first is hidden behind the
// previous tile's work. With no register cap (one CTA per SM) the tile body is the same code
// as k_tb_step's. The claim counter resets itself: the last CTA out zeroes it.

template <typename T, int RPT, int K>
struct PipeShape {
  static constexpr int W = TBVec<T>::W, ER = 8 * RPT, EC = 32 * W, PL = ER * EC, XCH = 9 * EC;
  static constexpr size_t STAGE = 3 * (size_t)PL * sizeof(T);  // Ex, Ey, Hz of the next tile
  static constexpr size_t CBUF = 4 * (size_t)PL * sizeof(T);   // cb_ex, cb_ey of two tiles
  static constexpr size_t XCHB = 2 * (size_t)XCH * sizeof(T);
  static constexpr uint32_t TX = (uint32_t)(5 * PL * sizeof(T));
  static constexpr size_t CPML = TBShape<T, RPT, K, KIND_XY>::SMEM;
  static constexpr size_t SMEM = 128 + (STAGE + CBUF + XCHB > CPML ? STAGE + CBUF + XCHB : CPML) + 16;
  static_assert((PL * sizeof(T)) % 128 == 0, "stage planes stay 128-byte aligned");
};

template <typename T, int RPT, int K, bool WITH_CPML = true>
__global__ void __launch_bounds__(TB_THREADS, 1)
k_tb_pipe(const __grid_constant__ TMAMaps maps, const __grid_constant__ SimArgs<T> a,
          const __grid_constant__ TBDst<T> dst, const int2* __restrict__ tiles, int n_inner, int n_pml,
          unsigned* __restrict__ ctr, const __grid_constant__ PhasePlan<T> ph,
          const __grid_constant__ PhasePlan<T> pe, int step_off) {
  using S = PipeShape<T, RPT, K>;
  constexpr int PL = S::PL;
  extern __shared__ __align__(128) unsigned char pipe_smem[];
  unsigned char* const base = pipe_smem + ((128u - (smem_addr(pipe_smem) & 127u)) & 127u);
  T* const stage = reinterpret_cast<T*>(base);
  T* const cbuf = reinterpret_cast<T*>(base + S::STAGE);
  T* const xch = reinterpret_cast<T*>(base + S::STAGE + S::CBUF);
  // past both layouts (a CPML tile uses the dynamic shared memory from its start)
  uint64_t* const mbar = reinterpret_cast<uint64_t*>(pipe_smem + S::SMEM - 16);
  __shared__ int s_next, s_pending, s_ok;
  const int tid = threadIdx.y * 32 + threadIdx.x;
  const int n_all = n_pml + n_inner;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto fetch = [&](int k_inner, int buf) {  // one thread: interior tile k_inner into stage, cb buffer buf
    const int2 t = tiles[k_inner];
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mbar)), "r"(S::TX)
                 : "memory");
    const int x = t.y - K, y = t.x - K;
    tma_load_tile(stage + 0 * PL, &maps.ex, x, y, mbar);
    tma_load_tile(stage + 1 * PL, &maps.ey, x, y, mbar);
    tma_load_tile(stage + 2 * PL, &maps.hz, x, y, mbar);
    tma_load_tile(cbuf + (2 * buf) * PL, &maps.cbx, x, y, mbar);
    tma_load_tile(cbuf + (2 * buf + 1) * PL, &maps.cby, x, y, mbar);
  };
  // claim the next tile; prefetch it into cb buffer `buf` when it is interior and `may_fetch`
  auto claim = [&](int buf, bool may_fetch) {
    if (tid == 0) {
      const int k = (int)atomicAdd(ctr, 1u);
      s_next = k;
      s_pending = 0;
      if (may_fetch && k >= n_pml && k < n_all) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fetch(k - n_pml, buf);
        s_pending = 1;
      }
    }
  };
  claim(0, true);
  __syncthreads();
  int cur = s_next, pending = s_pending, buf = 0;
  uint32_t parity = 0;
  while (cur < n_all) {
    if (WITH_CPML && cur < n_pml) {  // a CPML tile loads itself; nothing can be staged meanwhile
      const int2 raw = tiles[n_inner + cur];
      const int2 u = make_int2(raw.x & ((1 << KIND_SHIFT) - 1), raw.y);
      auto hook = [&]() { claim(buf, false); };
      switch (raw.x >> KIND_SHIFT) {
        case KIND_X: tb_tile<T, RPT, K, KIND_X>(a, dst, u, ph, pe, step_off, nullptr, nullptr, nullptr, hook); break;
        case KIND_Y: tb_tile<T, RPT, K, KIND_Y>(a, dst, u, ph, pe, step_off, nullptr, nullptr, nullptr, hook); break;
        default: tb_tile<T, RPT, K, KIND_XY>(a, dst, u, ph, pe, step_off, nullptr, nullptr, nullptr, hook); break;
      }
    } else {
      if (!pending && tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        fetch(cur - n_pml, buf);
      }
      if (tid == 0) s_ok = 1;
      __syncthreads();
      if (!mbar_wait_bounded(mbar, parity, a.flag)) s_ok = 0;
      parity ^= 1;
      if (!__syncthreads_and(s_ok)) break;  // the copy never landed: flagged, leave uniformly
      const int2 tile = tiles[cur - n_pml];
      auto hook = [&]() { claim(buf ^ 1, true); };
      tb_tile<T, RPT, K, KIND_INNER, true>(a, dst, tile, ph, pe, step_off, stage, cbuf + 2 * buf * PL, xch, hook);
      buf ^= 1;
    }
    __syncthreads();  // s_next, s_pending published; cb buffer and exchange rows free
    cur = s_next;
    pending = s_pending;
  }
  if (tid == 0) {  // the last CTA out resets the claim counter for the next launch
    __threadfence();
    if (atomicAdd(ctr + 1, 1u) == gridDim.x - 1) {
      ctr[0] = 0;
      ctr[1] = 0;
      __threadfence();
    }
  }
}

// ------------------------------------------------------------------------ host side

struct TBConfig {
  int dtype, RPT, K, NW;  // tile rows NW * RPT, columns 32 * W (128 for f32, 64 for f64), depth K, NW warps
};

// 40 x 128 tiles of 8 warps of 5 rows: 128 registers, two CTAs per SM, so one CTA's tile load
// overlaps the other's steps (9 % shorter launches than 48 x 128 tiles at one CTA per SM)
static constexpr TBConfig kDefault32 = {ETG_F32, 5, 4, 8};
// float64: 32 x 64 tiles (8 warps of 4 rows, two CTAs per SM) spill less under the 128-register
// cap than 40-row tiles and measured 4 % faster at 2024² (the FP64 pipe binds either way)
static constexpr TBConfig kDefault64 = {ETG_F64, 4, 2, 8};
static constexpr TBConfig kTmaDefault32 = {ETG_F32, 5, 4, 8};
static constexpr TBConfig kTmaDefault64 = {ETG_F64, 5, 2, 8};

struct TBState {
  TMAMaps maps[2];          // TMA descriptors of (fields A, cb) and (fields B, cb)
  bool maps_valid = false;
  int sms = 0;              // SMs of the device: one persistent CTA each
  int mode = -1;            // 0: interior + CPML kernels per launch, 1: persistent TMA kernel
  void* alt[7] = {};  // second buffer of each field / psi plane, same pitch
  size_t alt_bytes = 0;
  int2* tiles = nullptr;  // interior tiles first (those with sources, monitors or traces leading), then CPML tiles
  int n_inner = 0, n_pml = 0;
  int n_hot = 0;                 // leading interior tiles that hold a source, monitor or trace node
  std::vector<int4> hot_key;     // every hot rectangle seen since the grid was set (n_hot counts their tiles)
  TBConfig cfg = {0, 0, 0, 0};
  int nx = -1, ny = -1;
  bool tiles_valid = false;
  std::map<int64_t, cudaGraphExec_t> graphs;
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  cudaStream_t sides[4] = {};    // one branch per CPML kind, one for the interior tiles with a plan
  cudaEvent_t joins[4] = {};
  // per-kernel timing (ETG_OPT_TIMING 2): launches serialised on the main stream, no graphs
  bool profile = false;
  cudaEvent_t pev[7] = {};
  double prof_ms[2] = {};        // interior, CPML
  double prof_kind_ms[3] = {};   // CPML tiles of each kind launched alone: X, Y, XY
  int64_t prof_launches[2] = {};
  int64_t owned_cells[5] = {};   // output cells of one launch: lean interior tiles, every other tile
                                 // (CPML, interior with a plan), and per CPML kind
  int n_kind[6] = {};            // CPML tiles of each kind (the CPML list is sorted by kind), then
                                 // how many of each lead their kind with a source, monitor or trace
  unsigned* ctr = nullptr;       // persistent pipelined kernel: claim counters of the two launches
  // column segments of the lean interior tiles (k_tb_seg; tiles ER = 5K rows high): segs[0 ..
  // n_segs) = (first output row of the head, first column), then n_left lean tiles (r0, c0)
  // that no segment takes; the lean tiles of the tile list stay for the launches that cannot
  // use segments (traces, the TM variants, per-kernel timing)
  int2* segs = nullptr;
  int n_segs = 0, n_left = 0, seg_carried = 0;
};

TBState* tb_create() { return new TBState; }

static void tb_drop_graphs(TBState* tb) {
  for (auto& kv : tb->graphs) cudaGraphExecDestroy(kv.second);
  tb->graphs.clear();
}

void tb_destroy(TBState* tb) {
  if (!tb) return;
  tb_drop_graphs(tb);
  for (void* p : tb->alt) cudaFree(p);
  cudaFree(tb->tiles);
  cudaFree(tb->segs);
  cudaFree(tb->ctr);
  for (cudaEvent_t e : tb->pev)
    if (e) cudaEventDestroy(e);
  if (tb->side) cudaStreamDestroy(tb->side);
  for (int k = 0; k < 4; ++k) {
    if (tb->sides[k]) cudaStreamDestroy(tb->sides[k]);
    if (tb->joins[k]) cudaEventDestroy(tb->joins[k]);
  }
  if (tb->fork) cudaEventDestroy(tb->fork);
  if (tb->join) cudaEventDestroy(tb->join);
  delete tb;
}

int tb_segments(const TBState* tb) { return tb && tb->tiles_valid ? tb->n_segs : 0; }

void tb_invalidate(TBState* tb) {
  if (!tb) return;
  tb_drop_graphs(tb);
  tb->tiles_valid = false;
}

// Chosen by "auto": grids of at least 64 x 64 cells, in both precisions. In float64 GB300's
// FP64 pipe rather than HBM bounds the step; the blocked kernels still beat one step per
// launch there, halo recomputation included.
template <typename T>
bool tb_supported(int nx, int ny) {
  return nx >= 64 && ny >= 64;
}

template <typename T, int RPT, int K, bool PML, int NW = 8, bool PLAN = true, bool TMM = false>
static cudaError_t tb_launch_one(const SimArgs<T>& a, const TBDst<T>& d, const int2* tiles, int n,
                                 const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off,
                                 cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  k_tb_step<T, RPT, K, PML, NW, PLAN, TMM><<<n, dim3(32, NW), tb_smem<T, RPT, K, PML, NW>(), s>>>(a, d, tiles, ph,
                                                                                                pe, step_off);
  g_launches += 1;
  return cudaGetLastError();
}

// CPML tiles of one kind: the leading n_hot (sources, monitors, traces) with the plan code on
// `hot_stream`, the rest with the lean body on `stream`.
template <typename T, int RP, int K, int KIND, bool TMM = false>
static cudaError_t tb_launch_kind(const SimArgs<T>& a, const TBDst<T>& d, const int2* t, int n, int n_hot,
                                  const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off, cudaStream_t stream,
                                  cudaStream_t hot_stream) {
  constexpr size_t SMEM = TBShape<T, RP, K, KIND>::SMEM;
  if (n_hot) {
    k_tb_kind<T, RP, K, KIND, 8, true, TMM><<<n_hot, dim3(32, 8), SMEM, hot_stream>>>(a, d, t, ph, pe, step_off);
    g_launches += 1;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (n > n_hot) {
    k_tb_kind<T, RP, K, KIND, 8, false, TMM><<<n - n_hot, dim3(32, 8), SMEM, stream>>>(a, d, t + n_hot, ph, pe,
                                                                                      step_off);
    g_launches += 1;
    return cudaGetLastError();
  }
  return cudaSuccess;
}

// CPML tiles, one kernel per kind on its own side stream side[0..2], the tiles of each kind with
// a plan on side[3] (tiles sorted X, Y, XY from `tiles`; n_kind: three counts, three hot counts).
template <typename T, int RP, int K, bool TMM = false>
static cudaError_t tb_launch_kinds(const SimArgs<T>& a, const TBDst<T>& d, const int2* tiles, const int* n_kind,
                                   const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off,
                                   cudaStream_t const* side) {
  cudaError_t e = tb_launch_kind<T, RP, K, KIND_X, TMM>(a, d, tiles, n_kind[0], n_kind[3], ph, pe, step_off,
                                                        side[0], side[3]);
  tiles += n_kind[0];
  if (e == cudaSuccess)
    e = tb_launch_kind<T, RP, K, KIND_Y, TMM>(a, d, tiles, n_kind[1], n_kind[4], ph, pe, step_off, side[1],
                                              side[3]);
  tiles += n_kind[1];
  if (e == cudaSuccess)
    e = tb_launch_kind<T, RP, K, KIND_XY, TMM>(a, d, tiles, n_kind[2], n_kind[5], ph, pe, step_off, side[2],
                                               side[3]);
  return e;
}

template <typename T, int RPT, int K, int NW = 8, bool TMM = false>
static cudaError_t tb_launch_pair(TBState* tb, const SimArgs<T>& a, const TBDst<T>& d,
                                  const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off,
                                  cudaStream_t s) {
  constexpr int RP = RPT * NW / 8;  // CPML tiles: 8 warps over the same rows
  const int2* hot = tb->tiles;                 // interior tiles with sources, monitors or traces
  const int2* cold = tb->tiles + tb->n_hot;    // the other interior tiles: the lean kernel
  const int n_cold = tb->n_inner - tb->n_hot;
  // lean interior tiles as column segments (a head and carried tiles, k_tb_seg) plus the lean
  // tiles no segment takes; not with a trace (a segment recompute may skip tiles)
  bool segments = false;
  if constexpr (RPT * NW == 5 * K) segments = tb->n_segs > 0 && ph.trace.buf == nullptr;
  auto launch_segments = [&](cudaStream_t main) {
    cudaError_t e2 = cudaSuccess;
    if constexpr (RPT * NW == 5 * K) {
      k_tb_seg<T, RPT, K, NW, TMM><<<tb->n_segs, dim3(32, NW), tb_smem<T, RPT, K, false, NW>(), main>>>(
          a, d, tb->segs, tb->seg_carried, ph, pe, step_off);
      g_launches += 1;
      e2 = cudaGetLastError();
    }
    return e2;
  };
  auto launch_left = [&](cudaStream_t stream) {  // the lean tiles no segment takes
    return tb_launch_one<T, RPT, K, false, NW, false, TMM>(a, d, tb->segs + tb->n_segs, tb->n_left, ph, pe,
                                                           step_off, stream);
  };
  if (tb->profile) {  // one after the other on s, an event pair around each kernel
    cudaError_t e = cudaEventRecord(tb->pev[0], s);
    if (e == cudaSuccess)  // timed as the interior: the segments alone, or every lean tile
      e = segments ? launch_segments(s)
                   : tb_launch_one<T, RPT, K, false, NW, false, TMM>(a, d, cold, n_cold, ph, pe, step_off, s);
    const int2* t = tb->tiles + tb->n_inner;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
      int only[6] = {0, 0, 0, 0, 0, 0};
      only[k] = tb->n_kind[k];
      only[3 + k] = tb->n_kind[3 + k];
      e = cudaEventRecord(tb->pev[1 + k], s);
      if (e == cudaSuccess) {
        cudaStream_t ss[4] = {s, s, s, s};
        e = tb_launch_kinds<T, RP, K, TMM>(a, d, t, only, ph, pe, step_off, ss);
      }
      t += tb->n_kind[k];
    }
    if (e == cudaSuccess) e = cudaEventRecord(tb->pev[4], s);
    if (e == cudaSuccess) e = tb_launch_one<T, RPT, K, false, NW, true, TMM>(a, d, hot, tb->n_hot, ph, pe, step_off, s);
    if (e == cudaSuccess && segments) e = launch_left(s);  // with the other tiles
    if (e == cudaSuccess) e = cudaEventRecord(tb->pev[5], s);
    if (e == cudaSuccess) e = cudaEventSynchronize(tb->pev[5]);
    float m[5] = {};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = cudaEventElapsedTime(&m[k], tb->pev[k], tb->pev[k + 1]);
    tb->prof_ms[0] += m[0];
    tb->prof_ms[1] += m[1] + m[2] + m[3] + m[4];
    for (int k = 0; k < 3; ++k) tb->prof_kind_ms[k] += m[1 + k];
    tb->prof_launches[0] += n_cold > 0;
    tb->prof_launches[1] += tb->n_pml + tb->n_hot > 0;
    return e;
  }
  // CPML kinds and the interior tiles with a plan on four side branches, the other interior
  // tiles on the main stream (parallel graph nodes)
  cudaError_t e = cudaEventRecord(tb->fork, s);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(tb->sides[k], tb->fork, 0);
  if (e == cudaSuccess)
    e = tb_launch_kinds<T, RP, K, TMM>(a, d, tb->tiles + tb->n_inner, tb->n_kind, ph, pe, step_off, tb->sides);
  if (e == cudaSuccess)
    e = tb_launch_one<T, RPT, K, false, NW, true, TMM>(a, d, hot, tb->n_hot, ph, pe, step_off, tb->sides[3]);
  // (segments on the main stream, the lean tiles no segment takes beside the plan tiles)
  if (e == cudaSuccess && segments) e = launch_left(tb->sides[3]);
  if (e == cudaSuccess)
    e = segments ? launch_segments(s)
                 : tb_launch_one<T, RPT, K, false, NW, false, TMM>(a, d, cold, n_cold, ph, pe, step_off, s);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
    e = cudaEventRecord(tb->joins[k], tb->sides[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, tb->joins[k], 0);
  }
  return e;
}

template <typename T>
static SimArgs<T> swap_args(const SimArgs<T>& a, TBState* tb) {
  SimArgs<T> b = a;
  b.ex = (T*)tb->alt[ETG_EX];
  b.ey = (T*)tb->alt[ETG_EY];
  b.hz = (T*)tb->alt[ETG_HZ];
  b.psi_ex_y = (T*)tb->alt[ETG_PSI_EX_Y];
  b.psi_ey_x = (T*)tb->alt[ETG_PSI_EY_X];
  b.psi_hz_x = (T*)tb->alt[ETG_PSI_HZ_X];
  b.psi_hz_y = (T*)tb->alt[ETG_PSI_HZ_Y];
  return b;
}

template <typename T>
static TBDst<T> as_dst(const SimArgs<T>& a) {
  return TBDst<T>{a.ex, a.ey, a.hz, a.psi_ex_y, a.psi_ey_x, a.psi_hz_x, a.psi_hz_y};
}

// Two launches A -> B -> A covering 2K steps from step_off.
template <typename T, int RPT, int K, int NW = 8>
static cudaError_t tb_two(TBState* tb, const SimArgs<T>& a, const PhasePlan<T>& ph,
                          const PhasePlan<T>& pe, int step_off, cudaStream_t s) {
  const SimArgs<T> b = swap_args(a, tb);
  if (a.db_node) {  // TM mode: the kernels that read the per-node coefficient
    cudaError_t e = tb_launch_pair<T, RPT, K, NW, true>(tb, a, as_dst(b), ph, pe, step_off, s);
    if (e == cudaSuccess) e = tb_launch_pair<T, RPT, K, NW, true>(tb, b, as_dst(a), ph, pe, step_off + K, s);
    return e;
  }
  cudaError_t e = tb_launch_pair<T, RPT, K, NW>(tb, a, as_dst(b), ph, pe, step_off, s);
  if (e == cudaSuccess) e = tb_launch_pair<T, RPT, K, NW>(tb, b, as_dst(a), ph, pe, step_off + K, s);
  return e;
}

// Dynamic shared memory above 48 KB must be allowed per kernel, before any launch or capture.
template <typename T, int RPT, int K, int NW = 8>
static cudaError_t tb_attrs() {
  constexpr int RP = RPT * NW / 8;
  cudaError_t e = cudaSuccess;
#define ETG_STEP_ATTR(PL, TM)                                                                                   \
  if (e == cudaSuccess)                                                                                        \
    e = cudaFuncSetAttribute(k_tb_step<T, RPT, K, false, NW, PL, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)tb_smem<T, RPT, K, false, NW>());
#define ETG_KIND_ATTR(KD, PL, TM)                                                                               \
  if (e == cudaSuccess)                                                                                        \
    e = cudaFuncSetAttribute(k_tb_kind<T, RP, K, KD, 8, PL, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                             (int)TBShape<T, RP, K, KD>::SMEM);
  for (const bool tm : {false, true}) {
    // the TM variants (TMM) are separate kernels; both are allowed their shared memory up front
    if (tm) {
      ETG_STEP_ATTR(true, true)
      ETG_STEP_ATTR(false, true)
      ETG_KIND_ATTR(KIND_X, true, true)
      ETG_KIND_ATTR(KIND_X, false, true)
      ETG_KIND_ATTR(KIND_Y, true, true)
      ETG_KIND_ATTR(KIND_Y, false, true)
      ETG_KIND_ATTR(KIND_XY, true, true)
      ETG_KIND_ATTR(KIND_XY, false, true)
    } else {
      ETG_STEP_ATTR(true, false)
      ETG_STEP_ATTR(false, false)
      ETG_KIND_ATTR(KIND_X, true, false)
      ETG_KIND_ATTR(KIND_X, false, false)
      ETG_KIND_ATTR(KIND_Y, true, false)
      ETG_KIND_ATTR(KIND_Y, false, false)
      ETG_KIND_ATTR(KIND_XY, true, false)
      ETG_KIND_ATTR(KIND_XY, false, false)
    }
  }
#undef ETG_STEP_ATTR
#undef ETG_KIND_ATTR
  if constexpr (RPT * NW == 5 * K) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tb_seg<T, RPT, K, NW, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tb_smem<T, RPT, K, false, NW>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_tb_seg<T, RPT, K, NW, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tb_smem<T, RPT, K, false, NW>());
  }
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_tb_step<T, RPT * NW / 8, K, true, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)tb_smem<T, RPT * NW / 8, K, true, 8>());
  return e;
}

template <typename T>
struct TBFns {
  cudaError_t (*two)(TBState*, const SimArgs<T>&, const PhasePlan<T>&, const PhasePlan<T>&, int, cudaStream_t);
  cudaError_t (*attrs)();
};

// cuTensorMapEncodeTiled, looked up through the runtime (no link against libcuda).
static PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;

static int get_encoder() {
  if (g_encode_tiled) return ETG_OK;
  cudaDriverEntryPointQueryResult q;
  void* fn = nullptr;
  ETG_TRY_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
  ETG_REQUIRE(fn && q == cudaDriverEntryPointSuccess, ETG_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  g_encode_tiled = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  return ETG_OK;
}

// A 2D map over a pitched plane of nx + 2 rows, boxes of ER rows x EC columns, zeros outside.
template <typename T>
static int encode_plane(CUtensorMap* m, const void* base, int nx, int64_t P, int ER, int EC) {
  const cuuint64_t dims[2] = {(cuuint64_t)P, (cuuint64_t)(nx + 2)};
  const cuuint64_t strides[1] = {(cuuint64_t)(P * sizeof(T))};
  const cuuint32_t box[2] = {(cuuint32_t)EC, (cuuint32_t)ER};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = g_encode_tiled(m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                                    2, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  ETG_REQUIRE(r == CUDA_SUCCESS, ETG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return ETG_OK;
}

template <typename T, int RPT, int K>
static cudaError_t tma_attrs() {
  return cudaFuncSetAttribute(k_tb_tma<T, RPT, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)TMAShape<T, RPT, K>::SMEM);
}

// Two persistent launches A -> B -> A covering 2K steps from step_off.
template <typename T, int RPT, int K>
static cudaError_t tma_two(TBState* tb, const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
                           int step_off, cudaStream_t s) {
  using S = TMAShape<T, RPT, K>;
  const SimArgs<T> b = swap_args(a, tb);
  const int n = tb->n_inner + tb->n_pml, grid = std::min(n, 2 * tb->sms);
  k_tb_tma<T, RPT, K><<<grid, dim3(32, 8), S::SMEM, s>>>(tb->maps[0], a, as_dst(b), tb->tiles, tb->n_inner, n, ph, pe, step_off);
  k_tb_tma<T, RPT, K><<<grid, dim3(32, 8), S::SMEM, s>>>(tb->maps[1], b, as_dst(a), tb->tiles, tb->n_inner, n, ph, pe,
                                                         step_off + K);
  g_launches += 2;
  return cudaGetLastError();
}

template <typename T, int RPT, int K>
static cudaError_t pipe_attrs() {
  cudaError_t e = cudaFuncSetAttribute(k_tb_pipe<T, RPT, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)PipeShape<T, RPT, K>::SMEM);
  if (e == cudaSuccess) e = tb_attrs<T, RPT, K, 8>();  // the per-kind CPML kernels beside it
  return e;
}

// Two persistent pipelined launches A -> B -> A covering 2K steps from step_off, one CTA per SM
// on the interior tiles; the CPML tiles run as their per-kind kernels on the side branches,
// launched first, and the persistent CTAs take the SMs as those free them.
template <typename T, int RPT, int K>
static cudaError_t pipe_two(TBState* tb, const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
                            int step_off, cudaStream_t s) {
  using S = PipeShape<T, RPT, K>;
  const SimArgs<T> b = swap_args(a, tb);
  for (int half = 0; half < 2; ++half) {
    const SimArgs<T>& src = half ? b : a;
    const TBDst<T> d = as_dst(half ? a : b);
    const int off = step_off + half * K;
    cudaError_t e = cudaEventRecord(tb->fork, s);
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(tb->sides[k], tb->fork, 0);
    if (e == cudaSuccess) e = tb_launch_kinds<T, RPT, K>(src, d, tb->tiles + tb->n_inner, tb->n_kind, ph, pe, off, tb->sides);
    if (e != cudaSuccess) return e;
    k_tb_pipe<T, RPT, K, false><<<tb->sms, dim3(32, 8), S::SMEM, s>>>(tb->maps[half], src, d, tb->tiles, tb->n_inner, 0,
                                                                    tb->ctr + 2 * half, ph, pe, off);
    g_launches += 1;
    e = cudaGetLastError();
    for (int k = 0; k < 4 && e == cudaSuccess; ++k) {
      e = cudaEventRecord(tb->joins[k], tb->sides[k]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s, tb->joins[k], 0);
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Shapes of the persistent TMA kernel: two stages of five planes must fit 227 KB.
#define ETG_TMA_SHAPES_F32(X) X(ETG_F32, 5, 4)
#define ETG_TMA_SHAPES_F64(X) X(ETG_F64, 5, 2)

// Shapes of the persistent pipelined kernel: stage, two cb buffers and exchange rows must fit.
#define ETG_PIPE_SHAPES_F32(X) X(ETG_F32, 5, 4) X(ETG_F32, 6, 4)
#define ETG_PIPE_SHAPES_F64(X) X(ETG_F64, 4, 2) X(ETG_F64, 5, 2)

template <typename T>
static TBFns<T> pick(const TBConfig& c, int mode) {
#define ETG_TB_CASE(DT, R, KK, NWW) \
  if (c.dtype == DT && c.RPT == R && c.K == KK && c.NW == NWW) return {&tb_two<T, R, KK, NWW>, &tb_attrs<T, R, KK, NWW>};
#define ETG_TMA_CASE(DT, R, KK) \
  if (c.dtype == DT && c.RPT == R && c.K == KK && c.NW == 8) return {&tma_two<T, R, KK>, &tma_attrs<T, R, KK>};
#define ETG_PIPE_CASE(DT, R, KK) \
  if (c.dtype == DT && c.RPT == R && c.K == KK && c.NW == 8) return {&pipe_two<T, R, KK>, &pipe_attrs<T, R, KK>};
  if (mode == 2) {
    if constexpr (sizeof(T) == 4) {
      ETG_PIPE_SHAPES_F32(ETG_PIPE_CASE)
    } else {
      ETG_PIPE_SHAPES_F64(ETG_PIPE_CASE)
    }
  } else if (mode == 1) {
    if constexpr (sizeof(T) == 4) {
      ETG_TMA_SHAPES_F32(ETG_TMA_CASE)
    } else {
      ETG_TMA_SHAPES_F64(ETG_TMA_CASE)
    }
  } else {
    if constexpr (sizeof(T) == 4) {
      ETG_TB_SHAPES_F32(ETG_TB_CASE)
    } else {
      ETG_TB_SHAPES_F64(ETG_TB_CASE)
    }
  }
#undef ETG_TB_CASE
#undef ETG_TMA_CASE
#undef ETG_PIPE_CASE
  return {nullptr, nullptr};
}

static std::string shapes_text(int dtype, int mode) {
  std::string out;
#define ETG_TB_NAME(DT, R, KK) \
  if (DT == dtype) out += " " + std::to_string(8 * R) + "x" + std::to_string(DT == ETG_F32 ? 128 : 64) + "/K" + std::to_string(KK);
#define ETG_TB_NAME4(DT, R, KK, NWW)                                                                              \
  if (DT == dtype)                                                                                                \
    out += " " + std::to_string(NWW * R) + "x" + std::to_string(DT == ETG_F32 ? 128 : 64) + "/K" + std::to_string(KK) + \
           "/" + std::to_string(NWW) + "w";
  if (mode == 2) {
    ETG_PIPE_SHAPES_F32(ETG_TB_NAME)
    ETG_PIPE_SHAPES_F64(ETG_TB_NAME)
  } else if (mode == 1) {
    ETG_TMA_SHAPES_F32(ETG_TB_NAME)
    ETG_TMA_SHAPES_F64(ETG_TB_NAME)
  } else {
    ETG_TB_SHAPES_F32(ETG_TB_NAME4)
    ETG_TB_SHAPES_F64(ETG_TB_NAME4)
  }
#undef ETG_TB_NAME
#undef ETG_TB_NAME4
  return out;
}

// Interior tiles need their whole extended region in the unit rectangle and off the outer
// (PEC) edges.
// Tiles that hold a source node or a monitor node do extra work every step; they go first in
// their kind's list so that they start early instead of finishing last.
struct Hot {
  std::vector<int4> rects;  // x0, y0, x1, y1 (inclusive-exclusive) in cells
  bool hits(int r0, int c0, int rows, int cols) const {
    for (const int4& q : rects)
      if (q.x < r0 + rows && q.z > r0 && q.y < c0 + cols && q.w > c0) return true;
    return false;
  }
};

// With `hot`, the interior tiles whose extended region meets a hot rectangle lead the interior
// list and *n_hot counts them (the rest run the lean kernel, which has no source, monitor or
// trace code).
static void split_tiles(int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi, int ER, int EC,
                        int K, std::vector<int2>* tiles, int* n_inner, const Hot* hot = nullptr,
                        int* n_hot = nullptr, int* kind_hot = nullptr) {
  const int OR = ER - 2 * K, OC = EC - 2 * K;
  const int rlo = std::max(ux_lo, 1), rhi = std::min(ux_hi, nx), clo = std::max(uy_lo, 1), chi = std::min(uy_hi, ny);
  // First output column: shifted left by up to one tile width, in steps of a lane's W columns
  // (vector loads and TMA boxes stay 16-byte aligned), so that the fewest tile columns reach
  // the CPML columns. A CPML tile costs about two interior ones; ties keep column 0. At 2024
  // columns and 112-column tiles a shift of -52 leaves two CPML tile columns instead of three
  // (the third held the last 8 columns). Rows keep row 0: the tile kind is packed above them.
  int co = 0;
  {
    const int W = EC / 32;
    int best = 1 << 30;
    for (int off = 0; off > -OC; off -= W) {
      int cost = 0;
      for (int c0 = off; c0 <= ny; c0 += OC) cost += (c0 - K >= clo && c0 + OC + K <= chi) ? 1 : 2;
      if (cost < best) best = cost, co = off;
    }
  }
  std::vector<int2> inner, pml;
  for (int r0 = 0; r0 <= nx; r0 += OR)
    for (int c0 = co; c0 <= ny; c0 += OC) {
      const bool ux = r0 - K >= rlo && r0 + OR + K <= rhi, uy = c0 - K >= clo && c0 + OC + K <= chi;
      if (ux && uy) {
        inner.push_back(make_int2(r0, c0));
      } else {  // unit columns: CPML across rows only (X); unit rows: across columns only (Y)
        const int kind = uy ? KIND_X : ux ? KIND_Y : KIND_XY;
        pml.push_back(make_int2(r0 | (kind << KIND_SHIFT), c0));
      }
    }
  // CPML tiles grouped by kind (X, Y, XY), so that each kind is one contiguous range
  std::stable_sort(pml.begin(), pml.end(), [](int2 p, int2 q) { return (p.x >> KIND_SHIFT) < (q.x >> KIND_SHIFT); });
  if (n_hot) *n_hot = 0;
  if (kind_hot) kind_hot[0] = kind_hot[1] = kind_hot[2] = 0;
  if (hot) {
    auto first = [&](std::vector<int2>::iterator b, std::vector<int2>::iterator e) {
      return std::stable_partition(
          b, e, [&](int2 t) { return hot->hits((t.x & ((1 << KIND_SHIFT) - 1)) - K, t.y - K, ER, EC); });
    };
    const auto split = first(inner.begin(), inner.end());
    if (n_hot) *n_hot = (int)(split - inner.begin());
    for (int kind = KIND_X; kind <= KIND_XY; ++kind) {
      auto b = std::find_if(pml.begin(), pml.end(), [&](int2 t) { return (t.x >> KIND_SHIFT) == kind; });
      auto e = std::find_if(b, pml.end(), [&](int2 t) { return (t.x >> KIND_SHIFT) != kind; });
      const auto split = first(b, e);
      if (kind_hot) kind_hot[kind - 1] = (int)(split - b);
    }
  }
  *n_inner = (int)inner.size();
  inner.insert(inner.end(), pml.begin(), pml.end());
  *tiles = inner;
}

// Everything a tile must hold to need the per-step plan code: source nodes, monitor nodes and
// the trace box of an adjoint run.
template <typename T>
static Hot hot_of(const PhasePlan<T>& ph, const PhasePlan<T>& pe) {
  Hot h;
  for (const PhasePlan<T>* p : {&ph, &pe}) {
    for (int k = 0; k < p->n_src; ++k) h.rects.push_back(make_int4(p->src[k].i, p->src[k].j, p->src[k].i + 1, p->src[k].j + 1));
    for (int k = 0; k < p->n_mon; ++k) {
      const MonDesc<T>& m = p->mon[k];
      h.rects.push_back(make_int4(m.ix0, m.jy0, m.ix0 + m.nxm, m.jy0 + m.nym));
    }
  }
  const TraceDesc<T>& tr = ph.trace;
  if (tr.buf) h.rects.push_back(make_int4(tr.ti0, tr.tj0, tr.ti0 + tr.tnx, tr.tj0 + tr.tny));
  return h;
}

// Adds the rectangles of `add` that `into` lacks; true if any was new. A tile that once held a
// source, monitor or trace node keeps the kernel with the plan code: switching between runs
// with and without monitors or traces (an adjoint's forward pass and its recomputes) then
// reuses the tile list and its graphs. Past `cap` rectangles the union restarts from `add`.
bool tb_hot_union(std::vector<int4>* into, const std::vector<int4>& add, size_t cap) {
  bool grew = false;
  for (const int4& q : add) {
    bool have = false;
    for (const int4& r : *into) have |= r.x == q.x && r.y == q.y && r.z == q.z && r.w == q.w;
    if (!have) {
      into->push_back(q);
      grew = true;
    }
  }
  if (into->size() > cap) *into = add;
  return grew;
}

template <typename T>
static int tb_prepare(TBState* tb, const SimArgs<T>& a, const int64_t* opt, const Hot& hot) {
  const int dt = (int)sizeof(T);
  const int EC = 32 * TBVec<T>::W;
  const int mode = opt[ETG_OPT_KERNEL] == 3 ? 1 : opt[ETG_OPT_KERNEL] == 4 ? 2 : 0;
  TBConfig want = mode == 1 ? (dt == 4 ? kTmaDefault32 : kTmaDefault64) : (dt == 4 ? kDefault32 : kDefault64);
  if (opt[ETG_OPT_TB_DEPTH] > 0) want.K = (int)opt[ETG_OPT_TB_DEPTH];
  if (opt[ETG_OPT_TB_WARPS] > 0 && opt[ETG_OPT_TB_WARPS] != want.NW) {  // same rows, other split
    const int rows = want.RPT * want.NW, nw = (int)opt[ETG_OPT_TB_WARPS];
    if (opt[ETG_OPT_TILE_ROWS] == 0 && rows % nw != 0) {
      set_error("the default tile of %d rows does not split over %d warps: set ETG_OPT_TILE_ROWS too (have:%s)",
                rows, nw, shapes_text(dt, mode).c_str());
      return ETG_ERR_ARGUMENT;
    }
    want.RPT = rows / nw;
    want.NW = nw;
  }
  if (opt[ETG_OPT_TILE_ROWS] > 0) want.RPT = (int)(opt[ETG_OPT_TILE_ROWS] / want.NW);
  const bool cols_ok = opt[ETG_OPT_TILE_COLS] == 0 || opt[ETG_OPT_TILE_COLS] == EC;
  if (!cols_ok || opt[ETG_OPT_TILE_ROWS] % want.NW != 0 || !pick<T>(want, mode).two) {
    set_error("no compiled %s kernel with tile %lldx%lld and depth %d (have:%s)",
              mode == 1 ? "persistent TMA" : mode == 2 ? "persistent pipelined" : "temporally blocked",
              (long long)(opt[ETG_OPT_TILE_ROWS] ? opt[ETG_OPT_TILE_ROWS] : want.NW * want.RPT),
              (long long)(opt[ETG_OPT_TILE_COLS] ? opt[ETG_OPT_TILE_COLS] : EC), want.K,
              shapes_text(dt, mode).c_str());
    return ETG_ERR_ARGUMENT;
  }
  if (want.RPT != tb->cfg.RPT || want.K != tb->cfg.K || want.NW != tb->cfg.NW || want.dtype != tb->cfg.dtype ||
      mode != tb->mode) {
    tb_invalidate(tb);
    tb->cfg = want;
    tb->mode = mode;
    tb->maps_valid = false;
    ETG_TRY_CUDA(pick<T>(want, mode).attrs());
  }
  const size_t bytes = (size_t)(a.nx + 2) * a.P * sizeof(T);
  if (tb->alt_bytes != bytes) {
    tb_invalidate(tb);
    for (void*& p : tb->alt) {
      cudaFree(p);
      p = nullptr;
    }
    tb->maps_valid = false;
    for (void*& p : tb->alt) {
      if (cudaMalloc(&p, bytes) != cudaSuccess || cudaMemset(p, 0, bytes) != cudaSuccess) {
        cudaGetLastError();
        set_error("temporal blocking: cannot allocate %zu bytes for the second field buffer", bytes);
        return ETG_ERR_ALLOC;
      }
    }
    tb->alt_bytes = bytes;
  }
  if (!tb->side) {
    ETG_TRY_CUDA(cudaStreamCreateWithFlags(&tb->side, cudaStreamNonBlocking));
    ETG_TRY_CUDA(cudaEventCreateWithFlags(&tb->fork, cudaEventDisableTiming));
    ETG_TRY_CUDA(cudaEventCreateWithFlags(&tb->join, cudaEventDisableTiming));
    for (int k = 0; k < 4; ++k) {
      ETG_TRY_CUDA(cudaStreamCreateWithFlags(&tb->sides[k], cudaStreamNonBlocking));
      ETG_TRY_CUDA(cudaEventCreateWithFlags(&tb->joins[k], cudaEventDisableTiming));
    }
  }
  // the tiles holding sources, monitors or the trace decide which kernel runs a tile: split
  // again when one appears that the union of those seen so far does not hold
  if (tb->nx != a.nx || tb->ny != a.ny) tb->hot_key.clear();
  const bool grew = tb_hot_union(&tb->hot_key, hot.rects, 1024);
  if (!tb->tiles_valid || tb->nx != a.nx || tb->ny != a.ny || grew) {
    std::vector<int2> inner;
    Hot seen;
    seen.rects = tb->hot_key;
    split_tiles(a.nx, a.ny, a.ux_lo, a.ux_hi, a.uy_lo, a.uy_hi, tb->cfg.NW * tb->cfg.RPT, EC, tb->cfg.K, &inner,
                &tb->n_inner, &seen, &tb->n_hot, tb->n_kind + 3);
    tb->n_pml = (int)inner.size() - tb->n_inner;
    const int OR = tb->cfg.NW * tb->cfg.RPT - 2 * tb->cfg.K, OC = EC - 2 * tb->cfg.K;
    for (int64_t& c : tb->owned_cells) c = 0;
    for (int k = 0; k < 3; ++k) tb->n_kind[k] = 0;
    for (int q = 0; q < (int)inner.size(); ++q) {
      const int64_t r = std::max(0, std::min(OR, a.nx - tb_tile_row(inner[q]))),
                    c = std::max(0, std::min(OC, a.ny - inner[q].y));
      tb->owned_cells[q >= tb->n_hot && q < tb->n_inner ? 0 : 1] += r * c;
      if (q >= tb->n_inner) {
        const int kind = tb_tile_kind(inner[q]);
        tb->owned_cells[1 + kind] += r * c;
        tb->n_kind[kind - 1] += 1;
      }
    }
    cudaFree(tb->tiles);
    tb->tiles = nullptr;
    ETG_TRY_CUDA(cudaMalloc(&tb->tiles, inner.size() * sizeof(int2)));
    ETG_TRY_CUDA(cudaMemcpy(tb->tiles, inner.data(), inner.size() * sizeof(int2), cudaMemcpyHostToDevice));
    // column segments: runs of lean interior tiles in one column, five ordinary tiles' rows per
    // segment (a head and three carried tiles), when the tile is ER = 5K rows high
    cudaFree(tb->segs);
    tb->segs = nullptr;
    tb->n_segs = tb->n_left = tb->seg_carried = 0;
    if (tb->cfg.NW * tb->cfg.RPT == 5 * tb->cfg.K && mode == 0 && opt[ETG_OPT_TB_SEGMENTS] == 0) {
      if (tb->sms == 0) {
        int dev = 0;
        ETG_TRY_CUDA(cudaGetDevice(&dev));
        ETG_TRY_CUDA(cudaDeviceGetAttribute(&tb->sms, cudaDevAttrMultiProcessorCount, dev));
      }
      std::vector<int2> lean(inner.begin() + tb->n_hot, inner.begin() + tb->n_inner);
      std::sort(lean.begin(), lean.end(), [](int2 p, int2 q) { return p.y != q.y ? p.y < q.y : p.x < q.x; });
      std::vector<int2> segs, left;
      for (size_t b = 0; b < lean.size();) {
        size_t e = b + 1;  // a run: one column, rows OR apart
        while (e < lean.size() && lean[e].y == lean[b].y && lean[e].x == lean[e - 1].x + OR) ++e;
        const size_t n = e - b, g = n / 5;
        for (size_t q = 0; q < g; ++q) segs.push_back(lean[b + 5 * q]);
        for (size_t q = 5 * g; q < n; ++q) left.push_back(lean[b + q]);
        b = e;
      }
      // a segment holds four tiles' work in one CTA: with fewer segments than SMs the launch
      // cannot fill the GPU and the ordinary tiles are faster
      if ((int)segs.size() >= tb->sms && tb->sms > 0) {
        tb->n_segs = (int)segs.size();
        tb->n_left = (int)left.size();
        tb->seg_carried = 3;
        // per-kernel timing counts the segments as the interior, the leftover tiles with the rest
        const int64_t per_tile = (int64_t)OR * OC;  // an interior tile's output lies inside the grid
        tb->owned_cells[0] -= (int64_t)left.size() * per_tile;
        tb->owned_cells[1] += (int64_t)left.size() * per_tile;
        segs.insert(segs.end(), left.begin(), left.end());
        ETG_TRY_CUDA(cudaMalloc(&tb->segs, segs.size() * sizeof(int2)));
        ETG_TRY_CUDA(cudaMemcpy(tb->segs, segs.data(), segs.size() * sizeof(int2), cudaMemcpyHostToDevice));
      }
    }
    tb->nx = a.nx;
    tb->ny = a.ny;
    tb->tiles_valid = true;
    tb_drop_graphs(tb);
  }
  if (mode == 2 && !tb->ctr) {
    ETG_TRY_CUDA(cudaMalloc(&tb->ctr, 4 * sizeof(unsigned)));
    ETG_TRY_CUDA(cudaMemset(tb->ctr, 0, 4 * sizeof(unsigned)));
  }
  if (mode >= 1 && !tb->maps_valid) {
    ETG_REQUIRE(a.P >= EC && a.nx + 2 >= 8 * tb->cfg.RPT, ETG_ERR_ARGUMENT,
                "the persistent kernels need a grid of at least %d x %d cells", 8 * tb->cfg.RPT, EC);
    int rc = get_encoder();
    if (rc) return rc;
    int dev = 0;
    ETG_TRY_CUDA(cudaGetDevice(&dev));
    ETG_TRY_CUDA(cudaDeviceGetAttribute(&tb->sms, cudaDevAttrMultiProcessorCount, dev));
    const int ER = 8 * tb->cfg.RPT;
    const void* fa[3] = {a.ex, a.ey, a.hz};
    const void* fb[3] = {tb->alt[ETG_EX], tb->alt[ETG_EY], tb->alt[ETG_HZ]};
    for (int k = 0; k < 2; ++k) {
      const void* const* f = k == 0 ? fa : fb;
      TMAMaps& m = tb->maps[k];
      if ((rc = encode_plane<T>(&m.ex, f[0], a.nx, a.P, ER, EC)) || (rc = encode_plane<T>(&m.ey, f[1], a.nx, a.P, ER, EC)) ||
          (rc = encode_plane<T>(&m.hz, f[2], a.nx, a.P, ER, EC)) || (rc = encode_plane<T>(&m.cbx, a.cb_ex, a.nx, a.P, ER, EC)) ||
          (rc = encode_plane<T>(&m.cby, a.cb_ey, a.nx, a.P, ER, EC)))
        return rc;
    }
    tb->maps_valid = true;
  }
  return ETG_OK;
}

template <typename T>
int tb_advance(TBState* tb, const SimArgs<T>& a, const PhasePlan<T>& ph, const PhasePlan<T>& pe,
               int64_t n_steps, const int64_t* opt, cudaStream_t s) {
  int rc = tb_prepare<T>(tb, a, opt, hot_of(ph, pe));
  if (rc) return rc;
  tb->profile = opt[ETG_OPT_TIMING] == 2 && tb->mode == 0;
  if (tb->profile) {
    for (cudaEvent_t& e : tb->pev)
      if (!e) ETG_TRY_CUDA(cudaEventCreate(&e));
    tb->prof_ms[0] = tb->prof_ms[1] = 0;
    tb->prof_kind_ms[0] = tb->prof_kind_ms[1] = tb->prof_kind_ms[2] = 0;
    tb->prof_launches[0] = tb->prof_launches[1] = 0;
  }
  const auto two = pick<T>(tb->cfg, tb->mode).two;
  const int K = tb->cfg.K;
  const int64_t pairs = n_steps / (2 * K);
  const int64_t per_graph = std::max<int64_t>(1, opt[ETG_OPT_GRAPH_STEPS] / (2 * K));
  // a block: up to per_graph launch pairs, the DFT of the block's samples, the step counter
  auto block = [&](int64_t n_pairs) -> cudaError_t {
    cudaError_t e = cudaSuccess;
    for (int64_t p = 0; p < n_pairs && e == cudaSuccess; ++p) e = two(tb, a, ph, pe, (int)(2 * K * p), s);
    if (e == cudaSuccess) launch_dft_block<T>(a, ph, pe, (int)(2 * K * n_pairs), s);
    if (e == cudaSuccess) launch_step_add<T>(a, 2 * K * n_pairs, s);
    return e == cudaSuccess ? cudaGetLastError() : e;
  };
  int64_t done = 0;  // pairs launched
  if (opt[ETG_OPT_GRAPH_STEPS] > 0 && pairs >= per_graph && !tb->profile) {
    auto it = tb->graphs.find(per_graph);
    if (it == tb->graphs.end()) {
      cudaGraph_t graph;
      ETG_TRY_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const cudaError_t e = block(per_graph);
      cudaError_t e2 = cudaStreamEndCapture(s, &graph);
      ETG_REQUIRE(e == cudaSuccess && e2 == cudaSuccess, ETG_ERR_CUDA, "temporal-blocking graph capture failed: %s",
                  cudaGetErrorString(e != cudaSuccess ? e : e2));
      cudaGraphExec_t exec;
      e2 = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      ETG_REQUIRE(e2 == cudaSuccess, ETG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e2));
      it = tb->graphs.emplace(per_graph, exec).first;
    }
    for (; done + per_graph <= pairs; done += per_graph) {
      ETG_TRY_CUDA(cudaGraphLaunch(it->second, s));
      g_launches += 4 * per_graph + 2;
    }
  }
  while (done < pairs) {
    const int64_t c = std::min(per_graph, pairs - done);
    ETG_TRY_CUDA(block(c));
    done += c;
  }
  // the remainder (< 2K steps) with the one-step kernels, in place on the primary buffer
  const int64_t rem = n_steps - 2 * K * pairs;
  for (int64_t k = 0; k < rem; ++k) launch_step_plain<T>(a, ph, pe, (int)k, s);
  if (rem) launch_step_add<T>(a, rem, s);
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

void tb_kernel_timing(const TBState* tb, double* ms, int64_t* launches, int64_t* cells) {
  for (int k = 0; k < 5; ++k) {
    ms[k] = !tb ? 0 : k < 2 ? tb->prof_ms[k] : tb->prof_kind_ms[k - 2];
    launches[k] = !tb ? 0 : k < 2 ? tb->prof_launches[k] : (tb->n_kind[k - 2] ? tb->prof_launches[1] : 0);
    cells[k] = tb ? tb->owned_cells[k] : 0;
  }
}

template bool tb_supported<float>(int, int);
template bool tb_supported<double>(int, int);
template int tb_advance<float>(TBState*, const SimArgs<float>&, const PhasePlan<float>&,
                               const PhasePlan<float>&, int64_t, const int64_t*, cudaStream_t);
template int tb_advance<double>(TBState*, const SimArgs<double>&, const PhasePlan<double>&,
                                const PhasePlan<double>&, int64_t, const int64_t*, cudaStream_t);

}  // namespace etg

// ------------------------------------------------------------------------ default-shape helpers

namespace etg {

void tb_default_shape(int dtype, int* ER, int* EC, int* K, int kernel) {
  const TBConfig& c = kernel == 3 ? (dtype == ETG_F64 ? kTmaDefault64 : kTmaDefault32)
                                  : (dtype == ETG_F64 ? kDefault64 : kDefault32);
  *ER = 8 * c.RPT;
  *EC = dtype == ETG_F64 ? 64 : 128;
  *K = c.K;
}

void tb_tiles(int dtype, int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi,
              std::vector<int2>* tiles, int* n_inner) {
  int ER, EC, K;
  tb_default_shape(dtype, &ER, &EC, &K);
  split_tiles(nx, ny, ux_lo, ux_hi, uy_lo, uy_hi, ER, EC, K, tiles, n_inner);
}

template <typename T>
cudaError_t tb_default_launch(const SimArgs<T>& src, const SimArgs<T>& dst, const int2* tiles,
                              int n_inner, int n_pml, int step_off, cudaStream_t s) {
  constexpr TBConfig c = sizeof(T) == 4 ? kDefault32 : kDefault64;
  constexpr int RPT = c.RPT, K = c.K;
  static_assert(c.NW == 8, "the default shape is 8 warps");
  PhasePlan<T> none;
  memset(&none, 0, sizeof none);
  cudaError_t e = tb_attrs<T, RPT, K>();
  if (e == cudaSuccess)  // no sources, monitors or traces: every interior tile takes the lean kernel
    e = tb_launch_one<T, RPT, K, false, 8, false>(src, as_dst(dst), tiles, n_inner, none, none, step_off, s);
  if (e == cudaSuccess)
    e = tb_launch_one<T, RPT, K, true>(src, as_dst(dst), tiles + n_inner, n_pml, none, none, step_off, s);
  return e;
}

template cudaError_t tb_default_launch<float>(const SimArgs<float>&, const SimArgs<float>&, const int2*,
                                              int, int, int, cudaStream_t);
template cudaError_t tb_default_launch<double>(const SimArgs<double>&, const SimArgs<double>&,
                                               const int2*, int, int, int, cudaStream_t);

void tb_split_tiles(int nx, int ny, int ux_lo, int ux_hi, int uy_lo, int uy_hi, int ER, int EC, int K,
                    const std::vector<int4>& hot, std::vector<int2>* tiles, int* n_inner, int* n_hot,
                    int* kind_hot) {
  Hot h;
  h.rects = hot;
  split_tiles(nx, ny, ux_lo, ux_hi, uy_lo, uy_hi, ER, EC, K, tiles, n_inner, &h, n_hot, kind_hot);
}


}  // namespace etg

extern "C" int etg_debug_set_wait_tries(int64_t tries) {
  ETG_REQUIRE(tries <= (int64_t)etg::kWaitTries, ETG_ERR_ARGUMENT,
              "etg_debug_set_wait_tries: at most %u tries", etg::kWaitTries);
  const uint32_t v = tries < 0 ? etg::kWaitTries : (uint32_t)tries;
  ETG_TRY_CUDA(cudaMemcpyToSymbol(etg::g_wait_tries, &v, sizeof v));
  return ETG_OK;
}
