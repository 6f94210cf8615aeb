// Temporally blocked reverse sweep of the discrete adjoint: K reverse steps per launch.
//
// The one-step adjoint kernels (k_adj_re / k_adj_rh) have the data flow of the forward
// step mirrored: the lambda-Hz update RE(n) reads the E-node terms of its own node, of the
// node to its right (j+1) and of the node below (i+1); the lambda-E update RH(n) reads the
// H-cell terms of its own cell, of the cell to its left (j-1) and of the cell above (i-1).
// That is the forward's neighbour pattern, so the forward's tiling carries over: a CTA loads
// an output tile plus a K-cell halo, runs K reverse steps on chip with lambda Ex, Ey, Hz of
// RPT x W cells per thread in registers, and writes the output tile to the other buffer.
//
// Each node's transposed term (gx of an Ex node, gy of an Ey node, hx/hy of an Hz cell) is
// computed once per step by the thread that owns the node, which also advances the node's
// lambda-psi; neighbours get it by shuffle (columns) or through shared memory (a warp's first
// row of gy, last row of hy). The one-step kernels instead recompute a neighbour's term
// from a second lambda-psi buffer; both evaluate the same expressions in the same order on the
// same inputs, so the two sweeps give the same bits, and a sweep may mix them freely.
//
// dJ/dcb: the tiles over the design window record lambda E of the window at every step
// (float, one slot per step of the launch block); k_adj_grad then adds the block's terms in
// float64, one thread per node, in descending step order like the one-step kernel. Doing the
// float64 sums in the few window tiles themselves made them the stragglers of every launch. Adjoint sources (the transposed DFT
// monitors) come as per-node tables and are added wherever a tile holds the node.
#include <algorithm>
#include <cstring>

#include "etg_tb_adj.h"
#include "etg_tb_dev.cuh"

namespace etg {

// Tile kinds as in the forward kernels: 0 interior, 1 CPML across rows (X), 2 across
// columns (Y), 3 both; CPML tile lists carry the kind in bits 28-29 of the row (int2) or in .w.
constexpr int AKIND_X = 1, AKIND_Y = 2, AKIND_XY = 3, AKIND_SHIFT = 28;

template <typename T, int RPT, int K, int KIND>
struct AdjShape {
  static constexpr int W = TBVec<T>::W;
  static constexpr int ER = 8 * RPT, EC = 32 * W, OR = ER - 2 * K, OC = EC - 2 * K;
  static constexpr int PL = ER * EC;
  // cb_ex, cb_ey, then lambda psi_hz_x, psi_ey_x (x kinds), then psi_hz_y, psi_ex_y (y kinds)
  static constexpr int PLANES = 2 + ((KIND & AKIND_X) ? 2 : 0) + ((KIND & AKIND_Y) ? 2 : 0);
  static constexpr int XCH = 9 * EC;          // one exchange plane (gy or hy): 8 warps + a zero row
  static constexpr size_t SMEM = ((size_t)PLANES * PL + 2 * XCH) * sizeof(T);
  static constexpr int MIN_BLOCKS = 1;
  static_assert(K % W == 0, "the halo must keep vectors aligned");
  static_assert(OR > 0 && OC > 0, "halo larger than the tile");
};

// lambda += table value of step r for the nodes of `rel` this thread holds.
template <typename T, int RPT, int W>
__device__ __forceinline__ void adj_inject(const AdjSrc<T>* src, uint32_t rel, TBVec<T> (&ex)[RPT],
                                           TBVec<T> (&ey)[RPT], TBVec<T> (&hz)[RPT], int i0, int j0, int64_t r) {
  for (uint32_t m = rel; m; m &= m - 1) {
    const AdjSrc<T>& d = src[__ffs(m) - 1];
    const int t_o = d.i - i0, e_o = d.j - j0;
    if ((unsigned)t_o >= (unsigned)RPT || (unsigned)e_o >= (unsigned)W) continue;
    const T v = d.table[r];
#pragma unroll
    for (int t = 0; t < RPT; ++t)
#pragma unroll
      for (int e = 0; e < W; ++e)
        if (t == t_o && e == e_o) {
          if (d.comp == ETG_HZ) hz[t].v[e] = add(hz[t].v[e], v);
          else if (d.comp == ETG_EX) ex[t].v[e] = add(ex[t].v[e], v);
          else ey[t].v[e] = add(ey[t].v[e], v);
        }
  }
}

// CPML tiles of kind X (Y) have unit y (x) coefficients on every column (row) and advance
// lambda psi only on strip rows (columns), as the forward kernels do; XY tiles (corners)
// evaluate the one-step kernels' full expressions everywhere.
template <typename T, int RPT, int K, int KIND>
__device__ __forceinline__ void tb_adj_tile(const TBAdjArgs<T>& a, const int2 tile, int step_off) {
  using S = AdjShape<T, RPT, K, KIND>;
  using Vw = TBVec<T>;
  constexpr int W = S::W, ER = S::ER, EC = S::EC, PL = S::PL;
  constexpr bool PML = KIND != 0, PX = (KIND & AKIND_X) != 0, PY = (KIND & AKIND_Y) != 0;
  extern __shared__ __align__(16) unsigned char adj_smem[];
  T* const sCbx = reinterpret_cast<T*>(adj_smem);
  T* const sCby = sCbx + PL;
  T* const sPsiX = sCby + PL;                   // x kinds: lambda psi_hz_x, psi_ey_x
  T* const sPsiY = sPsiX + (PX ? 2 * PL : 0);   // y kinds: lambda psi_hz_y, psi_ex_y
  T* const sGy = sCbx + S::PLANES * PL;   // [k]: gy of warp k's first row; [8] = zeros
  T* const sHy = sGy + S::XCH;            // [k + 1]: hy of warp k's last row; [0] = zeros
  __shared__ uint32_t s_rel[2];

  const SimArgs<T>& s = a.s;
  const int lane = threadIdx.x, ty = threadIdx.y;
  const int R0 = tile.x - K, C0 = tile.y - K;
  const int nx = s.nx, ny = s.ny;
  const int64_t P = s.P;
  const int lj0 = W * lane, j0 = C0 + lj0;
  const int lr0 = RPT * ty, i0 = R0 + lr0;
  const bool lane_in = j0 >= 0 && j0 + W <= P;

  if (ty == 0) {
    auto hits = [&](const AdjSrc<T>* src, int n) {
      bool hit = false;
      if (lane < n) hit = src[lane].i >= R0 && src[lane].i < R0 + ER && src[lane].j >= C0 && src[lane].j < C0 + EC;
      return __ballot_sync(0xffffffffu, hit);
    };
    const uint32_t r0 = hits(a.hsrc, a.n_hsrc), r1 = hits(a.esrc, a.n_esrc);
    if (lane == 0) {
      s_rel[0] = r0;
      s_rel[1] = r1;
    }
    Vw z;
    z.zero();
    z.st(sHy + lj0);
  }
  if (ty == 7) {
    Vw z;
    z.zero();
    z.st(sGy + 8 * EC + lj0);
  }

  Vw lex[RPT], ley[RPT], lhz[RPT];
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = i0 + t;
    const bool in = lane_in && (unsigned)i <= (unsigned)nx;
    const int64_t g = (int64_t)i * P + j0;
    const int o = (lr0 + t) * EC + lj0;
    Vw cx, cy;
    if (in) {
      lex[t].ld(a.in[0] + g);
      ley[t].ld(a.in[1] + g);
      lhz[t].ld(a.in[2] + g);
      cx.ld(s.cb_ex + g);
      cy.ld(s.cb_ey + g);
    } else {
      lex[t].zero();
      ley[t].zero();
      lhz[t].zero();
      cx.zero();
      cy.zero();
    }
    cx.st(sCbx + o);
    cy.st(sCby + o);
    if (PX) {  // strip rows only (every row in corner tiles)
      Vw p0, p1;
      if (in && (KIND == AKIND_XY || i < s.xs_lo || i >= s.xs_hi)) {
        p0.ld(a.in[3] + g);  // lambda psi_hz_x
        p1.ld(a.in[6] + g);  // lambda psi_ey_x
      } else {
        p0.zero();
        p1.zero();
      }
      p0.st(sPsiX + o);
      p1.st(sPsiX + PL + o);
    }
    if (PY) {  // vectors meeting a strip column only
      Vw p0, p1;
      if (in && (KIND == AKIND_XY || j0 < s.ys_lo || j0 + W > s.ys_hi)) {
        p0.ld(a.in[4] + g);  // lambda psi_hz_y
        p1.ld(a.in[5] + g);  // lambda psi_ex_y
      } else {
        p0.zero();
        p1.zero();
      }
      p0.st(sPsiY + o);
      p1.st(sPsiY + PL + o);
    }
  }
  T byh[W], cyh[W], kyh[W], bye[W], cye[W], kye[W];
  T bxh[RPT], cxh[RPT], kxh[RPT], bxe[RPT], cxe[RPT], kxe[RPT];
  if (PY) {
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const int j = min(max(j0 + e, 0), ny - 1), je = min(max(j0 + e, 0), ny);
      byh[e] = s.by_h[j];
      cyh[e] = s.cy_h[j];
      kyh[e] = s.iky_h[j];
      bye[e] = s.by_e[je];
      cye[e] = s.cy_e[je];
      kye[e] = s.iky_e[je];
    }
  }
  if (PX) {
#pragma unroll
    for (int t = 0; t < RPT; ++t) {
      const int i = min(max(i0 + t, 0), nx - 1), ie = min(max(i0 + t, 0), nx);
      bxh[t] = s.bx_h[i];
      cxh[t] = s.cx_h[i];
      kxh[t] = s.ikx_h[i];
      bxe[t] = s.bx_e[ie];
      cxe[t] = s.cx_e[ie];
      kxe[t] = s.ikx_e[ie];
    }
  }
  const T db = s.db, idx = s.inv_dx, idy = s.inv_dy;
  const int64_t n_hi = a.ctl[0] - step_off, trace_n0 = a.ctl[1];

  // Transposed E update of the Ex node of cell (t, e): dJ/d(dHz/dy); advances lambda psi_ex_y.
  // (the one-step kernel's "iky·lc" with 1/kappa = 1 exactly is lc itself; the domain checks
  // a kind's rows or columns always pass are left out)
  // Each works on one row of this thread's W nodes with that row's lambda psi as one 16-byte
  // vector in registers (the nodes outside the strips keep theirs untouched).
  // Per-column tests (strip, domain) are selects between expressions computed for every
  // column, not branches, so the columns stay independent instructions; each selected
  // expression is the one-step kernel's.
  auto gx_row = [&](int t, const Vw& cb, T* out) {  // Ex nodes; advances lambda psi_ex_y
    Vw lp;
    if (PY) lp.ld(sPsiY + PL + (lr0 + t) * EC + lj0);
    const int i = i0 + t;
    const bool row_in = !PX || (i >= 0 && i < nx);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const T lc = mul(cb.v[e], lex[t].v[e]);
      const int j = j0 + e;
      if (!PML || !PY) {
        out[e] = row_in ? lc : zero<T>();  // 1/kappa = 1 exactly, no psi
      } else {
        const bool in = row_in && j >= 1 && j <= ny - 1, strip = j < s.ys_lo || j >= s.ys_hi;
        const T lpt = add(lp.v[e], lc);
        const T with_psi = add(mul(kye[e], lc), mul(cye[e], lpt)), without = mul(kye[e], lc);
        lp.v[e] = in && strip ? mul(bye[e], lpt) : lp.v[e];
        out[e] = !in ? zero<T>() : strip ? with_psi : without;
      }
    }
    if (PY) lp.st(sPsiY + PL + (lr0 + t) * EC + lj0);
  };
  auto gy_row = [&](int t, const Vw& cb, T* out) {  // Ey nodes; advances lambda psi_ey_x
    const int i = i0 + t;
    const bool xrow = PX && (i < s.xs_lo || i >= s.xs_hi);
    const bool row_in = !PX || (i >= 1 && i <= nx - 1);
    Vw lp;
    if (xrow) lp.ld(sPsiX + PL + (lr0 + t) * EC + lj0);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const T lc = -mul(cb.v[e], ley[t].v[e]);
      const int j = j0 + e;
      const bool in = row_in && (!PY || (j >= 0 && j < ny));
      if (!PML || !PX) {
        out[e] = in ? lc : zero<T>();
      } else if (xrow) {
        const T lpt = add(lp.v[e], lc);
        lp.v[e] = in ? mul(bxe[t], lpt) : lp.v[e];
        out[e] = in ? add(mul(kxe[t], lc), mul(cxe[t], lpt)) : zero<T>();
      } else {
        out[e] = in ? mul(kxe[t], lc) : zero<T>();
      }
    }
    if (xrow) lp.st(sPsiX + PL + (lr0 + t) * EC + lj0);
  };
  auto h_row = [&](int t, T* hx, T* hy) {  // Hz cells; advances lambda psi_hz_y, psi_hz_x
    const int i = i0 + t;
    const bool xrow = PX && (i < s.xs_lo || i >= s.xs_hi);
    const bool row_in = !PX || (i >= 0 && i < nx);
    Vw ly, lx;
    if (PY) ly.ld(sPsiY + (lr0 + t) * EC + lj0);
    if (xrow) lx.ld(sPsiX + (lr0 + t) * EC + lj0);
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const T la = mul(db, lhz[t].v[e]);
      const int j = j0 + e;
      if (!PML) {
        hx[e] = la;
        hy[e] = -la;
        continue;
      }
      const bool in = row_in && (!PY || (j >= 0 && j < ny));
      T vx, vy;
      if (!PY) {
        vx = la;
      } else {
        const bool strip = j < s.ys_lo || j >= s.ys_hi;
        const T lpt = add(ly.v[e], la);
        ly.v[e] = in && strip ? mul(byh[e], lpt) : ly.v[e];
        vx = strip ? add(mul(kyh[e], la), mul(cyh[e], lpt)) : mul(kyh[e], la);
      }
      if (!PX) {
        vy = -la;
      } else if (xrow) {
        const T lpt = sub(lx.v[e], la);
        lx.v[e] = in ? mul(bxh[t], lpt) : lx.v[e];
        vy = add(-mul(kxh[t], la), mul(cxh[t], lpt));
      } else {
        vy = -mul(kxh[t], la);
      }
      hx[e] = in ? vx : zero<T>();
      hy[e] = in ? vy : zero<T>();
    }
    if (PY) ly.st(sPsiY + (lr0 + t) * EC + lj0);
    if (xrow) lx.st(sPsiX + (lr0 + t) * EC + lj0);
  };

  __syncthreads();  // cb (and lambda psi) staged
  T gyf[W];         // gy of this warp's first row for the next RE
  {
    Vw cy;
    cy.ld(sCby + lr0 * EC + lj0);
#pragma unroll
    gy_row(0, cy, gyf);
    Vw g;
#pragma unroll
    for (int e = 0; e < W; ++e) g.v[e] = gyf[e];
    g.st(sGy + ty * EC + lj0);
  }
  __syncthreads();

  const uint32_t relH = s_rel[0], relE = s_rel[1];
  const int t_lo = max(0, K - lr0), t_hi = min(RPT, ER - K - lr0);
  const int e_lo = lj0 >= K ? 0 : W, e_hi = lj0 + W <= EC - K ? W : 0;
  const bool designed = a.ltrace && a.i0 <= tile.x + S::OR - 1 && a.i0 + a.nxd >= tile.x &&
                        a.j0 <= tile.y + S::OC - 1 && a.j0 + a.nyd >= tile.y;
  const int wy = a.nyd + 1;
  const int64_t wbox = (int64_t)(a.nxd + 1) * wy;

  for (int st = 0; st < K; ++st) {
    const int64_t n = n_hi - 1 - st;
    // ------------------------------------------------ lambda E of n + 1 on the window, for dJ/dcb
    if (designed) {
      T* lt = a.ltrace + (a.ctl[0] - 1 - n) * 2 * wbox;
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        const int di = i0 + t - a.i0;
        if (t < t_lo || t >= t_hi || (unsigned)di > (unsigned)a.nxd) continue;
#pragma unroll
        for (int e = 0; e < W; ++e) {
          const int dj = j0 + e - a.j0;
          if (e < e_lo || e >= e_hi || (unsigned)dj > (unsigned)a.nyd) continue;
          lt[(int64_t)di * wy + dj] = lex[t].v[e];
          lt[wbox + (int64_t)di * wy + dj] = ley[t].v[e];
        }
      }
    }
    // ------------------------------------------------ RE(n): lambda Hz
    {
      T gyc[W], gyn[W];
#pragma unroll
      for (int e = 0; e < W; ++e) gyc[e] = gyf[e];
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        T gxr[W];
        Vw cx;
        cx.ld(sCbx + (lr0 + t) * EC + lj0);
        gx_row(t, cx, gxr);
        // interior tiles leave lane 31 its own value: the tile's last column is K columns from
        // the output and a wrong value there moves one column per reverse step
        T gxn = __shfl_down_sync(0xffffffffu, gxr[0], 1);
        if (PML && lane == 31) gxn = zero<T>();
        if (t < RPT - 1) {
          Vw cy;
          cy.ld(sCby + (lr0 + t + 1) * EC + lj0);
          gy_row(t + 1, cy, gyn);
        } else {
          Vw g;
          g.ld(sGy + (ty + 1) * EC + lj0);
#pragma unroll
          for (int e = 0; e < W; ++e) gyn[e] = g.v[e];
        }
#pragma unroll
        for (int e = 0; e < W; ++e) {
          const T gx1 = e < W - 1 ? gxr[e + 1] : gxn;
          const T u = add(add(add(lhz[t].v[e], mul(idy, sub(gxr[e], gx1))), mul(idx, sub(gyc[e], gyn[e]))),
                          zero<T>());
          if (!PML) {
            lhz[t].v[e] = u;
          } else {
            const int i = i0 + t, j = j0 + e;
            if ((!PX || (i >= 0 && i < nx)) && (!PY || (j >= 0 && j < ny))) lhz[t].v[e] = u;
          }
          gyc[e] = gyn[e];
        }
      }
    }
    if (relH) adj_inject<T, RPT, W>(a.hsrc, relH, lex, ley, lhz, i0, j0, n);
    T hxl[W], hyl[W];  // this warp's last row, computed once and shared
    {
      Vw g;
      h_row(RPT - 1, hxl, hyl);
#pragma unroll
      for (int e = 0; e < W; ++e) g.v[e] = hyl[e];
      g.st(sHy + (ty + 1) * EC + lj0);
    }
    __syncthreads();
    // ------------------------------------------------ RH(n): lambda E (+ DFT-E term of n - 1)
    {
      T hyp[W];
      {
        Vw g;
        g.ld(sHy + ty * EC + lj0);
#pragma unroll
        for (int e = 0; e < W; ++e) hyp[e] = g.v[e];
      }
#pragma unroll
      for (int t = 0; t < RPT; ++t) {
        T hxc[W], hyc[W];
        if (t < RPT - 1) {
          h_row(t, hxc, hyc);
        } else {
#pragma unroll
          for (int e = 0; e < W; ++e) {
            hxc[e] = hxl[e];
            hyc[e] = hyl[e];
          }
        }
        T hxp = __shfl_up_sync(0xffffffffu, hxc[W - 1], 1);
        if (PML && lane == 0) hxp = zero<T>();  // lane 0 of interior tiles: as lane 31 above
#pragma unroll
        for (int e = 0; e < W; ++e) {
          const T hxleft = e > 0 ? hxc[e - 1] : hxp;
          T vx = add(lex[t].v[e], mul(idy, sub(hxleft, hxc[e])));
          T vy = add(ley[t].v[e], mul(idx, sub(hyp[e], hyc[e])));
          if (n >= 1) {
            vx = add(vx, zero<T>());
            vy = add(vy, zero<T>());
          }
          if (!PML) {
            lex[t].v[e] = vx;
            ley[t].v[e] = vy;
          } else {
            const int i = i0 + t, j = j0 + e;
            if ((!PX || (i >= 0 && i < nx)) && (!PY || (j >= 0 && j <= ny))) lex[t].v[e] = vx;
            if ((!PX || (i >= 0 && i <= nx)) && (!PY || (j >= 0 && j < ny))) ley[t].v[e] = vy;
          }
          hyp[e] = hyc[e];
        }
      }
    }
    if (relE && n >= 1) adj_inject<T, RPT, W>(a.esrc, relE, lex, ley, lhz, i0, j0, n - 1);
    if (st < K - 1) {
      Vw cy, g;
      cy.ld(sCby + lr0 * EC + lj0);
      gy_row(0, cy, gyf);
#pragma unroll
      for (int e = 0; e < W; ++e) g.v[e] = gyf[e];
      g.st(sGy + ty * EC + lj0);
    }
    __syncthreads();
  }

  if (e_lo != 0 || e_hi != W || !lane_in) return;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = i0 + t;
    if (t < t_lo || t >= t_hi || (unsigned)i > (unsigned)nx) continue;
    const int64_t g = (int64_t)i * P + j0;
    lex[t].st(a.out[0] + g);
    ley[t].st(a.out[1] + g);
    lhz[t].st(a.out[2] + g);
    // lambda psi stays +0 outside its strips in both buffers
    const int o = (lr0 + t) * EC + lj0;
    if (PX && (KIND == AKIND_XY || i < s.xs_lo || i >= s.xs_hi)) {
      Vw v;
      v.ld(sPsiX + o);
      v.st(a.out[3] + g);
      v.ld(sPsiX + PL + o);
      v.st(a.out[6] + g);
    }
    if (PY && (KIND == AKIND_XY || j0 < s.ys_lo || j0 + W > s.ys_hi)) {
      Vw v;
      v.ld(sPsiY + o);
      v.st(a.out[4] + g);
      v.ld(sPsiY + PL + o);
      v.st(a.out[5] + g);
    }
  }
}

template <typename T, int RPT, int K, bool PML>
constexpr size_t adj_smem() {
  return PML ? AdjShape<T, RPT, K, AKIND_XY>::SMEM : AdjShape<T, RPT, K, 0>::SMEM;
}

template <typename T, int RPT, int K, bool PML>
__device__ __forceinline__ void adj_dispatch(const TBAdjArgs<T>& a, int r0, int c0, int kind, int step_off) {
  const int2 u = make_int2(r0, c0);
  if (!PML) {
    tb_adj_tile<T, RPT, K, 0>(a, u, step_off);
    return;
  }
  switch (kind) {
    case AKIND_X: tb_adj_tile<T, RPT, K, AKIND_X>(a, u, step_off); break;
    case AKIND_Y: tb_adj_tile<T, RPT, K, AKIND_Y>(a, u, step_off); break;
    default: tb_adj_tile<T, RPT, K, AKIND_XY>(a, u, step_off); break;
  }
}

template <typename T, int RPT, int K, bool PML>
__global__ void __launch_bounds__(TB_THREADS, PML ? 1 : 2)
k_tb_adj(const __grid_constant__ TBAdjArgs<T> a, const int2* __restrict__ tiles, int step_off) {
  const int2 t = tiles[blockIdx.x];
  adj_dispatch<T, RPT, K, PML>(a, t.x & ((1 << AKIND_SHIFT) - 1), t.y, t.x >> AKIND_SHIFT, step_off);
}

template <typename T, int RPT, int K, bool PML>
__global__ void __launch_bounds__(TB_THREADS, PML ? 1 : 2)
k_tb_adj_batch(const TBAdjArgs<T>* __restrict__ args, const int4* __restrict__ tiles, int parity, int step_off) {
  const int4 t = tiles[blockIdx.x];  // simulation, r0, c0, kind
  adj_dispatch<T, RPT, K, PML>(args[2 * t.x + parity], t.y, t.z, t.w, step_off);
}

// One CPML kind per kernel (one tile body per kernel keeps each launch's code small).
template <typename T, int RPT, int K, int KIND>
__global__ void __launch_bounds__(TB_THREADS, 1)
k_tb_adj_kind(const __grid_constant__ TBAdjArgs<T> a, const int2* __restrict__ tiles, int step_off) {
  const int2 t = tiles[blockIdx.x];
  tb_adj_tile<T, RPT, K, KIND>(a, make_int2(t.x & ((1 << AKIND_SHIFT) - 1), t.y), step_off);
}

template <typename T, int RPT, int K, int KIND>
__global__ void __launch_bounds__(TB_THREADS, 1)
k_tb_adj_batch_kind(const TBAdjArgs<T>* __restrict__ args, const int4* __restrict__ tiles, int parity, int step_off) {
  const int4 t = tiles[blockIdx.x];  // simulation, r0, c0, kind
  tb_adj_tile<T, RPT, K, KIND>(args[2 * t.x + parity], make_int2(t.y, t.z), step_off);
}

__global__ void k_adj_ctl_add(int64_t* ctl, int64_t delta) { ctl[0] += delta; }

// dJ/dcb += the window's terms of steps ctl[0]-1 … ctl[0]-n_slots for design blockIdx.y
// (args[stride * design]): one thread per Ex or Ey node, float64, in descending step order —
// the one-step kernel's additions in its order, spread over the whole GPU.
template <typename T>
__global__ void k_adj_grad(const TBAdjArgs<T>* __restrict__ args, int stride, int n_slots) {
  const TBAdjArgs<T>& a = args[stride * blockIdx.y];
  const int nx_ = a.nxd, ny_ = a.nyd, wy = ny_ + 1;
  const int64_t n_ex = (int64_t)nx_ * wy, n_ey = (int64_t)(nx_ + 1) * ny_;
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_ex + n_ey) return;
  const bool is_ex = q < n_ex;
  const int64_t qq = is_ex ? q : q - n_ex;
  const int di = (int)(is_ex ? qq / wy : qq / ny_), dj = (int)(is_ex ? qq % wy : qq % ny_);
  const int ri = di + a.i0 - a.ti0, rj = dj + a.j0 - a.tj0;
  const int64_t wbox = (int64_t)(nx_ + 1) * wy, top = a.ctl[0], n0 = a.ctl[1];
  double* const gp = is_ex ? a.gx + qq : a.gy + qq;
  double g = *gp;
  const T idx = a.s.inv_dx, idy = a.s.inv_dy;
  for (int k = 0; k < n_slots; ++k) {
    const T* tr = a.trace + (top - 1 - k - n0) * a.tnx * a.tny;
    const T* lt = a.ltrace + (int64_t)k * 2 * wbox;
    if (is_ex) {
      const T c = add(mul(sub(tr[ri * a.tny + rj], tr[ri * a.tny + rj - 1]), idy), zero<T>());
      g += (double)lt[(int64_t)di * wy + dj] * (double)c;
    } else {
      const T c = add(mul(sub(tr[ri * a.tny + rj], tr[(ri - 1) * a.tny + rj]), idx), zero<T>());
      g -= (double)lt[wbox + (int64_t)di * wy + dj] * (double)c;
    }
  }
  *gp = g;
}

template <typename T>
void tb_adj_grad(const TBAdjArgs<T>* args, int stride, int n_designs, int64_t max_nodes, int n_slots, cudaStream_t s) {
  const dim3 grid((unsigned)((max_nodes + 127) / 128), (unsigned)n_designs);
  k_adj_grad<T><<<grid, 128, 0, s>>>(args, stride, n_slots);
  g_launches += 1;
}

template void tb_adj_grad<float>(const TBAdjArgs<float>*, int, int, int64_t, int, cudaStream_t);
template void tb_adj_grad<double>(const TBAdjArgs<double>*, int, int, int64_t, int, cudaStream_t);

void tb_adj_ctl_add(int64_t* ctl, int64_t delta, cudaStream_t s) {
  k_adj_ctl_add<<<1, 1, 0, s>>>(ctl, delta);
  g_launches += 1;
}

// ------------------------------------------------------------------------ host side

// Compiled shapes: 40-row tiles of 8 steps (float32: the forward's deep tile, which also
// shortened the reverse sweep, config-5 batch 1.87 s to 1.78 s) and of 2 steps (float64).
template <typename T>
struct AdjCfg;
template <>
struct AdjCfg<float> {
  static constexpr int RPT = 5, K = 8;
};
template <>
struct AdjCfg<double> {
  static constexpr int RPT = 5, K = 2;
};

void tb_adj_shape(int dtype, int* ER, int* EC, int* K) {
  if (dtype == ETG_F64) {
    *ER = 8 * AdjCfg<double>::RPT;
    *EC = 32 * TBVec<double>::W;
    *K = AdjCfg<double>::K;
  } else {
    *ER = 8 * AdjCfg<float>::RPT;
    *EC = 32 * TBVec<float>::W;
    *K = AdjCfg<float>::K;
  }
}

template <typename T>
int tb_adj_attrs() {
  constexpr int RPT = AdjCfg<T>::RPT, K = AdjCfg<T>::K;
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj<T, RPT, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)adj_smem<T, RPT, K, false>()));
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj<T, RPT, K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)adj_smem<T, RPT, K, true>()));
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj_batch<T, RPT, K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)adj_smem<T, RPT, K, false>()));
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj_batch<T, RPT, K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)adj_smem<T, RPT, K, true>()));
#define ETG_ADJ_KIND_ATTR(KD)                                                                             \
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj_kind<T, RPT, K, KD>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                    (int)AdjShape<T, RPT, K, KD>::SMEM));                                  \
  ETG_TRY_CUDA(cudaFuncSetAttribute(k_tb_adj_batch_kind<T, RPT, K, KD>,                                  \
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)AdjShape<T, RPT, K, KD>::SMEM));
  ETG_ADJ_KIND_ATTR(AKIND_X)
  ETG_ADJ_KIND_ATTR(AKIND_Y)
  ETG_ADJ_KIND_ATTR(AKIND_XY)
#undef ETG_ADJ_KIND_ATTR
  return ETG_OK;
}

template <typename T>
int tb_adj_launch(const TBAdjArgs<T>& a, const int2* tiles, int n_inner, const int* n_kind, int step_off,
                  cudaStream_t main, const cudaStream_t* sides, cudaEvent_t fork, const cudaEvent_t* joins) {
  constexpr int RPT = AdjCfg<T>::RPT, K = AdjCfg<T>::K;
  ETG_TRY_CUDA(cudaEventRecord(fork, main));
  for (int k = 0; k < 3; ++k) ETG_TRY_CUDA(cudaStreamWaitEvent(sides[k], fork, 0));
  const int2* t = tiles + n_inner;
  if (n_kind[0]) {
    k_tb_adj_kind<T, RPT, K, AKIND_X><<<n_kind[0], dim3(32, 8), AdjShape<T, RPT, K, AKIND_X>::SMEM, sides[0]>>>(
        a, t, step_off);
    g_launches += 1;
  }
  t += n_kind[0];
  if (n_kind[1]) {
    k_tb_adj_kind<T, RPT, K, AKIND_Y><<<n_kind[1], dim3(32, 8), AdjShape<T, RPT, K, AKIND_Y>::SMEM, sides[1]>>>(
        a, t, step_off);
    g_launches += 1;
  }
  t += n_kind[1];
  if (n_kind[2]) {
    k_tb_adj_kind<T, RPT, K, AKIND_XY><<<n_kind[2], dim3(32, 8), AdjShape<T, RPT, K, AKIND_XY>::SMEM, sides[2]>>>(
        a, t, step_off);
    g_launches += 1;
  }
  if (n_inner) {
    k_tb_adj<T, RPT, K, false><<<n_inner, dim3(32, 8), adj_smem<T, RPT, K, false>(), main>>>(a, tiles, step_off);
    g_launches += 1;
  }
  ETG_TRY_CUDA(cudaGetLastError());
  for (int k = 0; k < 3; ++k) {
    ETG_TRY_CUDA(cudaEventRecord(joins[k], sides[k]));
    ETG_TRY_CUDA(cudaStreamWaitEvent(main, joins[k], 0));
  }
  return ETG_OK;
}

template <typename T>
int tb_adj_batch_launch(const TBAdjArgs<T>* args, const int4* tiles, int n_inner, const int* n_kind, int parity,
                        int step_off, cudaStream_t main, const cudaStream_t* sides, cudaEvent_t fork,
                        const cudaEvent_t* joins) {
  constexpr int RPT = AdjCfg<T>::RPT, K = AdjCfg<T>::K;
  ETG_TRY_CUDA(cudaEventRecord(fork, main));
  for (int k = 0; k < 3; ++k) ETG_TRY_CUDA(cudaStreamWaitEvent(sides[k], fork, 0));
  const int4* t = tiles + n_inner;
  if (n_kind[0]) {
    k_tb_adj_batch_kind<T, RPT, K, AKIND_X><<<n_kind[0], dim3(32, 8), AdjShape<T, RPT, K, AKIND_X>::SMEM, sides[0]>>>(
        args, t, parity, step_off);
    g_launches += 1;
  }
  t += n_kind[0];
  if (n_kind[1]) {
    k_tb_adj_batch_kind<T, RPT, K, AKIND_Y><<<n_kind[1], dim3(32, 8), AdjShape<T, RPT, K, AKIND_Y>::SMEM, sides[1]>>>(
        args, t, parity, step_off);
    g_launches += 1;
  }
  t += n_kind[1];
  if (n_kind[2]) {
    k_tb_adj_batch_kind<T, RPT, K, AKIND_XY>
        <<<n_kind[2], dim3(32, 8), AdjShape<T, RPT, K, AKIND_XY>::SMEM, sides[2]>>>(args, t, parity, step_off);
    g_launches += 1;
  }
  if (n_inner) {
    k_tb_adj_batch<T, RPT, K, false><<<n_inner, dim3(32, 8), adj_smem<T, RPT, K, false>(), main>>>(args, tiles, parity,
                                                                                                 step_off);
    g_launches += 1;
  }
  ETG_TRY_CUDA(cudaGetLastError());
  for (int k = 0; k < 3; ++k) {
    ETG_TRY_CUDA(cudaEventRecord(joins[k], sides[k]));
    ETG_TRY_CUDA(cudaStreamWaitEvent(main, joins[k], 0));
  }
  return ETG_OK;
}

template int tb_adj_attrs<float>();
template int tb_adj_attrs<double>();
template int tb_adj_launch<float>(const TBAdjArgs<float>&, const int2*, int, const int*, int, cudaStream_t,
                                  const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);
template int tb_adj_launch<double>(const TBAdjArgs<double>&, const int2*, int, const int*, int, cudaStream_t,
                                   const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);
template int tb_adj_batch_launch<float>(const TBAdjArgs<float>*, const int4*, int, const int*, int, int,
                                        cudaStream_t, const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);
template int tb_adj_batch_launch<double>(const TBAdjArgs<double>*, const int4*, int, const int*, int, int,
                                         cudaStream_t, const cudaStream_t*, cudaEvent_t, const cudaEvent_t*);

}  // namespace etg
