// Device side of the temporally blocked kernels, shared by the single-grid launches
// (etg_tb.cu) and the batched ones (etg_tb_batch.cu): tile shapes, the tile body that advances
// one extended tile K steps, and the kernels that run it. The two translation units compile in
// parallel. See etg_tb.cu for the tiling and the exactness argument.
#pragma once

#include "etg_tb.h"
#include "etg_tb_dev.cuh"

namespace etg {

// Tile kinds: KIND_INNER (unit rectangle, lean update), KIND_X (CPML only across rows: the
// tile's columns are unit), KIND_Y (CPML only across columns), KIND_XY (both: corners).
constexpr int KIND_INNER = 0, KIND_X = 1, KIND_Y = 2, KIND_XY = 3;
constexpr int KIND_SHIFT = 28;  // CPML tile lists carry the kind in bits 28-29 of the row

template <typename T, int RPT, int K, int KIND, int NW = 8>
struct TBShape {
  static constexpr int W = TBVec<T>::W;
  static constexpr int ER = NW * RPT, EC = 32 * W, OR = ER - 2 * K, OC = EC - 2 * K;
  static constexpr int PL = ER * EC;                    // one plane: cb or psi
  // cb_ex, cb_ey, then psi_hz_x, psi_ey_x (x kinds), then psi_hz_y, psi_ex_y (y kinds)
  static constexpr int PLANES = 2 + ((KIND & KIND_X) ? 2 : 0) + ((KIND & KIND_Y) ? 2 : 0);
  static constexpr int XCH = (NW + 1) * EC;             // one exchange buffer: NW warps + a zero row
  static constexpr size_t SMEM = ((size_t)PLANES * PL + 2 * XCH) * sizeof(T);
  static constexpr int MIN_BLOCKS = KIND || NW != 8 ? 1 : (RPT <= 5 ? 2 : 1);
  static_assert(K % W == 0, "the halo must keep vectors aligned");
  static_assert(OR > 0 && OC > 0, "halo larger than the tile");
};

// acc[f, k] += value * phasor[n, f] for the owned output cells of this thread inside monitor d.
template <typename T, int RPT, int W>
__device__ __forceinline__ void tb_dft(const MonDesc<T>& d, const TBVec<T> (&val)[RPT], int i0, int j0,
                                       int t_lo, int t_hi, int e_lo, int e_hi, int64_t r) {
  const int64_t nodes = (int64_t)d.nxm * d.nym;
  const T* phr = d.table + 2 * r * d.n_f;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    if (t < t_lo || t >= t_hi) continue;
    const unsigned di = (unsigned)(i0 + t - d.ix0);
    if (di >= (unsigned)d.nxm) continue;
#pragma unroll
    for (int e = 0; e < W; ++e) {
      if (e < e_lo || e >= e_hi) continue;
      const unsigned dj = (unsigned)(j0 + e - d.jy0);
      if (dj >= (unsigned)d.nym) continue;
      dft_node(d.acc, nodes, (int64_t)di * d.nym + dj, phr, d.n_f, val[t].v[e]);
    }
  }
}

// Record this thread's owned nodes of monitor d in its sample slot (summed by k_dft_block).
template <typename T, int RPT, int W>
__device__ __forceinline__ void tb_sample(const MonDesc<T>& d, const TBVec<T> (&val)[RPT], int i0, int j0,
                                          int t_lo, int t_hi, int e_lo, int e_hi, int slot) {
  const int64_t nodes = (int64_t)d.nxm * d.nym;
  T* out = d.samp + (int64_t)slot * nodes;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    if (t < t_lo || t >= t_hi) continue;
    const unsigned di = (unsigned)(i0 + t - d.ix0);
    if (di >= (unsigned)d.nxm) continue;
#pragma unroll
    for (int e = 0; e < W; ++e) {
      if (e < e_lo || e >= e_hi) continue;
      const unsigned dj = (unsigned)(j0 + e - d.jy0);
      if (dj < (unsigned)d.nym) out[(int64_t)di * d.nym + dj] = val[t].v[e];
    }
  }
}

// Subtract the deltas of step n of the sources whose node this thread holds.
template <typename T, int RPT, int W>
__device__ __forceinline__ void tb_inject(const PhasePlan<T>& p, uint32_t rel, TBVec<T> (&ex)[RPT],
                                          TBVec<T> (&ey)[RPT], TBVec<T> (&hz)[RPT], int i0, int j0,
                                          int64_t n, int* flag) {
  for (uint32_t m = rel; m; m &= m - 1) {
    const SrcDesc<T>& d = p.src[__ffs(m) - 1];
    const int t_o = d.i - i0, e_o = d.j - j0;
    if ((unsigned)t_o >= (unsigned)RPT || (unsigned)e_o >= (unsigned)W) continue;
    const int64_t r = n - d.n0;
    if (r < 0 || r >= d.rows) {
      atomicOr(flag, ERRBIT_TABLE);
      continue;
    }
    const T delta = d.table[r * d.stride];
#pragma unroll
    for (int t = 0; t < RPT; ++t)
#pragma unroll
      for (int e = 0; e < W; ++e)
        if (t == t_o && e == e_o) {
          if (d.comp == ETG_HZ) hz[t].v[e] = sub(hz[t].v[e], delta);
          else if (d.comp == ETG_EX) ex[t].v[e] = sub(ex[t].v[e], delta);
          else ey[t].v[e] = sub(ey[t].v[e], delta);
        }
  }
}

// One CTA, one tile: load the extended tile, advance it K steps, write the output tile.
//
// CPML tiles come in three kinds. In an X tile every column of the extended region lies in
// the unit range of the y coefficients, so the y terms take the lean form; rows outside the
// x strips have no psi and their x terms reduce to d·(1/kappa) + 0 (b·0 + 0·d = +0 for
// finite d), a test that is uniform across a warp (one warp, one row); only strip rows read
// and write psi. Y tiles have unit x terms; their strip columns fall across the lanes of every
// warp, so all columns evaluate the full y expression (psi = +0 outside the strips gives the
// same bits) and only the psi store is predicated. XY tiles (corners) run the full
// expression everywhere. All give Etalon's bits.
struct TBNoHook {
  __device__ void operator()() const {}
};

// Carried tiles (CARRY): consecutive interior tiles of one column, stepped by one CTA. Each
// tile stores, at every step s, the new Hz of its local row ER - K - 1 in half `par` of a
// shared carry buffer (the row just above the next tile's first output row); a carried tile
// has no top halo (its first local row is its first output row) and takes that row's Hz at
// step s from the other half for the Ey update of its first row, the one value from above a
// step needs. The values are the ones a top halo would have recomputed, bit for bit.
template <typename T>
struct TBCarry {
  int par = 0;            // the half this tile writes; a carried tile reads the other
  bool carried = false;   // false: an ordinary tile with its K-row top halo (a segment's head)
};

// STAGED (interior tiles of the persistent kernel): Ex, Ey, Hz of the extended tile are
// already in shared memory at `stage` (three planes) and cb at `cb_s` (two planes), placed
// there by TMA; the exchange rows live at `xch_s`. `after_load` runs on every thread right
// after the barrier that ends the load phase, when the stage is free again.
// PLAN false (interior tiles that hold no source node, no monitor node and no trace cell):
// the tile skips the per-step source, monitor and trace code altogether. Without it the
// interior kernel fits 128 registers with no spills, which makes its launches about 15 %
// shorter; the tile lists put such tiles after the others, so each part is its own launch.
// TMM (the dual TE run of a TM run, compiled separately so TE kernels carry none of it):
// cb_ex and cb_ey both hold dt/mu0, so the cb_ey plane of the tile carries the per-node
// Hz-position coefficient (SimArgs::db_node) and the Ey update reads the cb_ex plane.
template <typename T, int RPT, int K, int KIND, bool STAGED = false, typename Hook = TBNoHook, int NW = 8,
          bool PLAN = true, bool TMM = false, bool CARRY = false>
__device__ __forceinline__ void tb_tile(const SimArgs<T>& a, const TBDst<T>& dst, const int2 tile,
                                        const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off,
                                        const T* stage = nullptr, T* cb_s = nullptr, T* xch_s = nullptr,
                                        Hook after_load = Hook(), const TBCarry<T>& carry = TBCarry<T>()) {
  using S = TBShape<T, RPT, K, KIND, NW>;
  using Vw = TBVec<T>;
  constexpr int W = S::W, ER = S::ER, EC = S::EC, PL = S::PL;
  constexpr bool PML = KIND != KIND_INNER, PX = (KIND & KIND_X) != 0, PY = (KIND & KIND_Y) != 0;
  static_assert(!STAGED || !PML, "only interior tiles are staged");
  static_assert(!STAGED || NW == 8, "the staged layout is for 8 warps");
  static_assert(!CARRY || (!PML && !PLAN && !STAGED), "carried tiles are lean interior tiles");
  extern __shared__ __align__(16) unsigned char tb_smem[];
  T* const sCbx = STAGED ? cb_s : reinterpret_cast<T*>(tb_smem);
  T* const sCby = sCbx + PL;
  T* const sPsiX = sCby + PL;                    // x kinds: psi_hz_x, psi_ey_x
  T* const sPsiY = sPsiX + (PX ? 2 * PL : 0);    // y kinds: psi_hz_y, psi_ex_y
  T* const sHzX = STAGED ? xch_s : sCbx + S::PLANES * PL;  // [k = ty + 1]: last-row Hz of warp ty; [0] = zeros
  T* const sEyX = sHzX + S::XCH;                 // [k = ty]: first-row Ey of warp ty; [NW] = zeros
  __shared__ uint32_t s_rel[4];  // relevant plan entries: H sources, E sources, H monitors, E monitors

  if constexpr (!STAGED) {
    // recompute of an adjoint segment: a tile whose output lies farther (in cells) from the
    // trace box than the steps left in the segment cannot change the trace and does nothing
    // (the whole CTA leaves before its first barrier). Values move one cell per step, so the
    // tiles still stepped read exact halos: each of their cells was within the cone one launch
    // earlier. 2K + 2 cells of margin.
    const TraceDesc<T>& tr = ph.trace;
    if (tr.buf && tr.cone) {
      const int di = max(0, max(tr.ti0 - (tile.x + S::OR - 1), tile.x - (tr.ti0 + tr.tnx - 1)));
      const int dj = max(0, max(tr.tj0 - (tile.y + S::OC - 1), tile.y - (tr.tj0 + tr.tny - 1)));
      const int64_t left = tr.n0 + tr.rows - (*a.step + step_off);
      if ((int64_t)max(di, dj) > left + 2 * K + 2) return;
    }
  }
  const int lane = threadIdx.x, ty = threadIdx.y;
  // carried tiles: one carry buffer per CTA, kept from tile to tile (declared here, once for
  // both forms of the step loop below)
  __shared__ __align__(16) T carry_s[CARRY ? 2 * K * EC : 1];
  const int TH = (CARRY && carry.carried) ? 0 : K;  // top halo rows
  const int R0 = tile.x - TH, C0 = tile.y - K;     // global cell of local (0, 0); C0 % W == 0
  const int nx = a.nx, ny = a.ny;
  const int64_t P = a.P;
  const int lj0 = W * lane, j0 = C0 + lj0;     // this lane's first column, local and global
  const int lr0 = RPT * ty, i0 = R0 + lr0;     // this warp's first row, local and global
  const bool lane_in = j0 >= 0 && j0 + W <= P;

  if (PLAN && ty == 0) {  // which plan entries touch this tile (sources: extended region; monitors: output)
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
        hit = d.ix0 < tile.x + S::OR && d.ix0 + d.nxm > tile.x && d.jy0 < tile.y + S::OC &&
              d.jy0 + d.nym > tile.y;
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
  if (ty == 0) {
    Vw z;
    z.zero();
    z.st(sHzX + lj0);  // the row above the tile
  }
  if (ty == NW - 1) {
    Vw z;
    z.zero();
    z.st(sEyX + NW * EC + lj0);  // the row below the tile
  }

  static_assert(!(TMM && STAGED), "the staged kernels take cb by TMA, not the TM coefficient");
  constexpr bool tm = TMM;
  // load the extended tile: fields to registers, cb (and psi) to shared memory
  Vw ex[RPT], ey[RPT], hz[RPT];
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int li = lr0 + t, i = i0 + t;
    const bool in = lane_in && (unsigned)i <= (unsigned)nx;
    const int64_t g = (int64_t)i * P + j0;
    const int o = li * EC + lj0;
    if (STAGED) {  // the whole extended region of an interior tile lies inside the grid
      ex[t].ld(stage + 0 * PL + o);
      ey[t].ld(stage + 1 * PL + o);
      hz[t].ld(stage + 2 * PL + o);
      continue;
    }
    Vw cx, cy;
    if (in) {
      ex[t].ld(a.ex + g);
      ey[t].ld(a.ey + g);
      hz[t].ld(a.hz + g);
      cx.ld(a.cb_ex + g);
      cy.ld((tm ? a.db_node : a.cb_ey) + g);
    } else {
      ex[t].zero();
      ey[t].zero();
      hz[t].zero();
      cx.zero();
      cy.zero();
    }
    cx.st(sCbx + o);
    cy.st(sCby + o);
    // psi only where it can be non-zero: x strips for psi_*_x, y strips for psi_*_y; the
    // update never reads it anywhere else (XY tiles read all of it)
    if (PX) {
      Vw p0, p1;
      if (in && (KIND == KIND_XY || i < a.xs_lo || i >= a.xs_hi)) {
        p0.ld(a.psi_hz_x + g);
        p1.ld(a.psi_ey_x + g);
      } else {
        p0.zero();
        p1.zero();
      }
      p0.st(sPsiX + o);
      p1.st(sPsiX + PL + o);
    }
    if (PY) {
      Vw p0, p1;
      if (in && (KIND == KIND_XY || j0 < a.ys_lo || j0 + W > a.ys_hi)) {
        p0.ld(a.psi_hz_y + g);
        p1.ld(a.psi_ex_y + g);
      } else {
        p0.zero();
        p1.zero();
      }
      p0.st(sPsiY + o);
      p1.st(sPsiY + PL + o);
    }
  }
  ey[0].st(sEyX + ty * EC + lj0);
  // CPML tiles: this thread's profiles in registers (columns per lane, rows per warp)
  T byh[W], cyh[W], kyh[W], bye[W], cye[W], kye[W];
  T bxh[RPT], cxh[RPT], kxh[RPT], bxe[RPT], cxe[RPT], kxe[RPT];
  if (PY) {
#pragma unroll
    for (int e = 0; e < W; ++e) {
      const int j = min(max(j0 + e, 0), ny - 1), je = min(max(j0 + e, 0), ny);
      byh[e] = a.by_h[j];
      cyh[e] = a.cy_h[j];
      kyh[e] = a.iky_h[j];
      bye[e] = a.by_e[je];
      cye[e] = a.cy_e[je];
      kye[e] = a.iky_e[je];
    }
  }
  if (PX) {
#pragma unroll
    for (int t = 0; t < RPT; ++t) {
      const int i = min(max(i0 + t, 0), nx - 1), ie = min(max(i0 + t, 0), nx);
      bxh[t] = a.bx_h[i];
      cxh[t] = a.cx_h[i];
      kxh[t] = a.ikx_h[i];
      bxe[t] = a.bx_e[ie];
      cxe[t] = a.cx_e[ie];
      kxe[t] = a.ikx_e[ie];
    }
  }
  // Interior tiles drop the "+ psi" of each curl term (psi = +0 there, and x + 0 only turns
  // -0 into +0) when no Ex, Ey or Hz value of the extended tile is -0. That is exact: a sum
  // is -0 only when both terms are and a difference x - y only when x is -0 and y is +0, so
  // a field that is not -0 never becomes -0 (updates, sources), and with the curl terms taken
  // as they are, results differ from the "+ 0" form only in the sign of a zero increment,
  // which leaves a field that is not -0 unchanged. Tiles that load a -0 (uploaded state) keep
  // the adds.
  bool keep0 = true;
  if (!PML) {
    bool nz = false;
#pragma unroll
    for (int t = 0; t < RPT; ++t)
#pragma unroll
      for (int e = 0; e < W; ++e)
        nz |= is_neg_zero(ex[t].v[e]) | is_neg_zero(ey[t].v[e]) | is_neg_zero(hz[t].v[e]);
    keep0 = __syncthreads_or(nz) != 0;
  } else {
    __syncthreads();
  }
  after_load();
  const uint32_t relSrcH = PLAN ? s_rel[0] : 0u, relSrcE = PLAN ? s_rel[1] : 0u;
  const uint32_t relMonH = PLAN ? s_rel[2] : 0u, relMonE = PLAN ? s_rel[3] : 0u;
  const int64_t n_base = *a.step + step_off;
  const T db = a.db, idx = a.inv_dx, idy = a.inv_dy;
  // owned output cells of this thread: rows t in [t_lo, t_hi), columns e in [e_lo, e_hi)
  const int t_lo = max(0, TH - lr0), t_hi = min(RPT, ER - K - lr0);
  const int e_lo = lj0 >= K ? 0 : W, e_hi = lj0 + W <= EC - K ? W : 0;
  const bool traced = PLAN && ph.trace.buf && ph.trace.ti0 < tile.x + S::OR && ph.trace.ti0 + ph.trace.tnx > tile.x &&
                      ph.trace.tj0 < tile.y + S::OC && ph.trace.tj0 + ph.trace.tny > tile.y;

  auto steps = [&](auto keep_tag) {
    constexpr bool KEEP0 = decltype(keep_tag)::value;
    auto body = [&](const int s) {
      const int64_t n = n_base + s;
      // ---------------------------------------------------------------- H half step
      {
        Vw eyb;
        eyb.ld(sEyX + (ty + 1) * EC + lj0);  // Ey of the row below this warp
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          // lane 31 takes its own value in interior tiles: the last column of the extended
          // tile is K columns from the output and its error moves one column per step
          T exr = __shfl_down_sync(0xffffffffu, ex[t].v[0], 1);
          if (PML && lane == 31) exr = zero<T>();
          Vw dbr;  // this row's Hz-position coefficients: the scalar db, or per node in TM mode
          if constexpr (tm) dbr.ld(sCby + (lr0 + t) * EC + lj0);
          else dbr.fill(db);
          // CPML tiles: this row's psi as one 16-byte vector per lane. Outside the strips psi
          // is +0 and its update b*0 + 0*d is +0 again, so whole vectors go back unchanged there.
          const int ir = i0 + t;
          const bool xrow = KIND == KIND_XY || ir < a.xs_lo || ir >= a.xs_hi;
          Vw pyv, pxv;
          if (PY) pyv.ld(sPsiY + (lr0 + t) * EC + lj0);
          if (PX && xrow) pxv.ld(sPsiX + (lr0 + t) * EC + lj0);
#pragma unroll
          for (int e = 0; e < W; ++e) {
            const T exn = e < W - 1 ? ex[t].v[e + 1] : exr;
            const T eyn = t < RPT - 1 ? ey[t + 1].v[e] : eyb.v[e];
            const T dex_dy = mul(sub(exn, ex[t].v[e]), idy);
            const T dey_dx = mul(sub(eyn, ey[t].v[e]), idx);
            if (!PML) {
              if (KEEP0) hz[t].v[e] = add(hz[t].v[e], mul(dbr.v[e], sub(add(dex_dy, zero<T>()), add(dey_dx, zero<T>()))));
              else hz[t].v[e] = add(hz[t].v[e], mul(dbr.v[e], sub(dex_dy, dey_dx)));
            } else {
              // computed for every cell and kept only inside the domain: selects, not branches,
              // so the cells of a row stay independent instructions
              const int i = ir, j = j0 + e;
              const bool in = (!PX || (i >= 0 && i < nx)) && (!PY || (j >= 0 && j < ny));
              T ty_ = add(dex_dy, zero<T>()), tx_ = add(dey_dx, zero<T>());
              if (PY) {  // every column alike: no divergence between strip and other lanes
                const T py = add(mul(byh[e], pyv.v[e]), mul(cyh[e], dex_dy));
                pyv.v[e] = in ? py : pyv.v[e];
                ty_ = add(mul(dex_dy, kyh[e]), py);
              }
              if (PX) {
                if (xrow) {
                  const T px = add(mul(bxh[t], pxv.v[e]), mul(cxh[t], dey_dx));
                  pxv.v[e] = in ? px : pxv.v[e];
                  tx_ = add(mul(dey_dx, kxh[t]), px);
                } else {
                  tx_ = add(mul(dey_dx, kxh[t]), zero<T>());
                }
              }
              const T h1 = add(hz[t].v[e], mul(dbr.v[e], sub(ty_, tx_)));
              hz[t].v[e] = in ? h1 : hz[t].v[e];
            }
          }
          if (PY) pyv.st(sPsiY + (lr0 + t) * EC + lj0);
          if (PX && xrow) pxv.st(sPsiX + (lr0 + t) * EC + lj0);
        }
      }
      if (relSrcH) tb_inject<T, RPT, W>(ph, relSrcH, ex, ey, hz, i0, j0, n, a.flag);
      if (relMonH) {  // DFT of H at (n + 1/2) dt, owned nodes only (or their samples)
        for (uint32_t m = relMonH; m; m &= m - 1) {
          const MonDesc<T>& d = ph.mon[__ffs(m) - 1];
          const int64_t r = n - d.n0;
          if (d.samp) tb_sample<T, RPT, W>(d, hz, i0, j0, t_lo, t_hi, e_lo, e_hi, step_off + s);
          else if (r < 0 || r >= d.rows) atomicOr(a.flag, ERRBIT_TABLE);
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
      if constexpr (CARRY) {
        constexpr int CR = ER - K - 1;  // the row above the next tile
        if (ty == CR / RPT) hz[CR % RPT].st(carry_s + (carry.par * K + s) * EC + lj0);
        if (carry.carried && ty == 0) {  // the row above this tile, from the previous tile
          Vw c;
          c.ld(carry_s + ((carry.par ^ 1) * K + s) * EC + lj0);
          c.st(sHzX + lj0);
        }
      }
      __syncthreads();
      // ---------------------------------------------------------------- E half step
      {
        Vw hza;
        hza.ld(sHzX + ty * EC + lj0);  // Hz of the row above this warp
#pragma unroll
        for (int t = 0; t < RPT; ++t) {
          T hzl = __shfl_up_sync(0xffffffffu, hz[t].v[W - 1], 1);
          if (PML && lane == 0) hzl = zero<T>();  // lane 0 of interior tiles: as lane 31 above
          Vw cx, cy;
          cx.ld(sCbx + (lr0 + t) * EC + lj0);
          cy.ld((tm ? sCbx : sCby) + (lr0 + t) * EC + lj0);
          const int ir = i0 + t;
          const bool xrow = KIND == KIND_XY || ir < a.xs_lo || ir >= a.xs_hi;
          Vw pyv, pxv;  // psi_ex_y, psi_ey_x of this row (CPML tiles)
          if (PY) pyv.ld(sPsiY + PL + (lr0 + t) * EC + lj0);
          if (PX && xrow) pxv.ld(sPsiX + PL + (lr0 + t) * EC + lj0);
#pragma unroll
          for (int e = 0; e < W; ++e) {
            const T hzp = e > 0 ? hz[t].v[e - 1] : hzl;
            const T hzu = t > 0 ? hz[t - 1].v[e] : hza.v[e];
            const T dy = mul(sub(hz[t].v[e], hzp), idy);
            const T dx = mul(sub(hz[t].v[e], hzu), idx);
            if (!PML) {
              if (KEEP0) {
                ex[t].v[e] = add(ex[t].v[e], mul(cx.v[e], add(dy, zero<T>())));
                ey[t].v[e] = sub(ey[t].v[e], mul(cy.v[e], add(dx, zero<T>())));
              } else {
                ex[t].v[e] = add(ex[t].v[e], mul(cx.v[e], dy));
                ey[t].v[e] = sub(ey[t].v[e], mul(cy.v[e], dx));
              }
            } else {  // as in the H half step: every cell computed, kept inside the domain
              const int i = ir, j = j0 + e;
              const bool in_x = (!PX || (i >= 0 && i < nx)) && (!PY || (j >= 1 && j <= ny - 1));
              const bool in_y = (!PX || (i >= 1 && i <= nx - 1)) && (!PY || (j >= 0 && j < ny));
              {
                T term = add(dy, zero<T>());
                if (PY) {  // every column alike
                  const T p = add(mul(bye[e], pyv.v[e]), mul(cye[e], dy));
                  pyv.v[e] = in_x ? p : pyv.v[e];
                  term = add(mul(dy, kye[e]), p);
                }
                const T e1 = add(ex[t].v[e], mul(cx.v[e], term));
                ex[t].v[e] = in_x ? e1 : ex[t].v[e];
              }
              {
                T term = add(dx, zero<T>());
                if (PX) {
                  if (xrow) {
                    const T p = add(mul(bxe[t], pxv.v[e]), mul(cxe[t], dx));
                    pxv.v[e] = in_y ? p : pxv.v[e];
                    term = add(mul(dx, kxe[t]), p);
                  } else {
                    term = add(mul(dx, kxe[t]), zero<T>());
                  }
                }
                const T e1 = sub(ey[t].v[e], mul(cy.v[e], term));
                ey[t].v[e] = in_y ? e1 : ey[t].v[e];
              }
            }
          }
          if (PY) pyv.st(sPsiY + PL + (lr0 + t) * EC + lj0);
          if (PX && xrow) pxv.st(sPsiX + PL + (lr0 + t) * EC + lj0);
        }
      }
      if (relSrcE) tb_inject<T, RPT, W>(pe, relSrcE, ex, ey, hz, i0, j0, n, a.flag);
      if (relMonE) {  // DFT of E at (n + 1) dt (or the samples)
        for (uint32_t m = relMonE; m; m &= m - 1) {
          const MonDesc<T>& d = pe.mon[__ffs(m) - 1];
          const int64_t r = n - d.n0;
          if (d.samp) {
            if (d.comp == ETG_EX) tb_sample<T, RPT, W>(d, ex, i0, j0, t_lo, t_hi, e_lo, e_hi, step_off + s);
            else tb_sample<T, RPT, W>(d, ey, i0, j0, t_lo, t_hi, e_lo, e_hi, step_off + s);
          } else if (r < 0 || r >= d.rows) {
            atomicOr(a.flag, ERRBIT_TABLE);
          } else if (d.comp == ETG_EX) {
            tb_dft<T, RPT, W>(d, ex, i0, j0, t_lo, t_hi, e_lo, e_hi, r);
          } else {
            tb_dft<T, RPT, W>(d, ey, i0, j0, t_lo, t_hi, e_lo, e_hi, r);
          }
        }
      }
      ey[0].st(sEyX + ty * EC + lj0);
      __syncthreads();
    };
    if constexpr (KEEP0 && !PML) {  // the rare path (a -0 was loaded) stays small in the instruction cache
#pragma unroll 1
      for (int s = 0; s < K; ++s) body(s);
    } else {
      for (int s = 0; s < K; ++s) body(s);
    }
  };
  if constexpr (PML) {
    steps(BoolTag<true>{});
  } else if (keep0) {
    steps(BoolTag<true>{});
  } else {
    steps(BoolTag<false>{});
  }

  // write the output tile (vectors lie wholly inside or outside it: K, OC are multiples of W)
  if (e_lo != 0 || e_hi != W || !lane_in) return;
#pragma unroll
  for (int t = 0; t < RPT; ++t) {
    const int i = i0 + t;
    if (t < t_lo || t >= t_hi || (unsigned)i > (unsigned)nx) continue;
    const int64_t g = (int64_t)i * P + j0;
    ex[t].st(dst.ex + g);
    ey[t].st(dst.ey + g);
    hz[t].st(dst.hz + g);
    // psi stays +0 outside its strips in both buffers: strip rows (x) and vectors that
    // meet a strip column (y) are written, as whole vectors
    const int o = (lr0 + t) * EC + lj0;
    if (PX && (KIND == KIND_XY || i < a.xs_lo || i >= a.xs_hi)) {
      Vw v;
      v.ld(sPsiX + o);
      v.st(dst.psi_hz_x + g);
      v.ld(sPsiX + PL + o);
      v.st(dst.psi_ey_x + g);
    }
    if (PY && (KIND == KIND_XY || j0 < a.ys_lo || j0 + W > a.ys_hi)) {
      Vw v;
      v.ld(sPsiY + o);
      v.st(dst.psi_hz_y + g);
      v.ld(sPsiY + PL + o);
      v.st(dst.psi_ex_y + g);
    }
  }
}

// Shared memory of a launch of the interior kernel (PML false) or the CPML kernel (the
// largest CPML kind).
template <typename T, int RPT, int K, bool PML, int NW = 8>
constexpr size_t tb_smem() {
  return TBShape<T, RPT, K, PML ? KIND_XY : KIND_INNER, NW>::SMEM;
}

template <typename T, int RPT, int K, int KIND, int NW, bool PLAN = true, bool TMM = false>
__device__ __forceinline__ void tb_tile_nw(const SimArgs<T>& a, const TBDst<T>& dst, const int2 tile,
                                           const PhasePlan<T>& ph, const PhasePlan<T>& pe, int step_off) {
  tb_tile<T, RPT, K, KIND, false, TBNoHook, NW, PLAN, TMM>(a, dst, tile, ph, pe, step_off);
}

template <typename T, int RPT, int K, bool PML, int NW = 8, bool PLAN = true, bool TMM = false>
__global__ void __launch_bounds__(32 * NW, TBShape<T, RPT, K, PML ? KIND_XY : KIND_INNER, NW>::MIN_BLOCKS)
k_tb_step(const __grid_constant__ SimArgs<T> a, const __grid_constant__ TBDst<T> dst,
          const int2* __restrict__ tiles, const __grid_constant__ PhasePlan<T> ph,
          const __grid_constant__ PhasePlan<T> pe, int step_off) {
  const int2 t = tiles[blockIdx.x];
  if (!PML) {
    tb_tile_nw<T, RPT, K, KIND_INNER, NW, PLAN, TMM>(a, dst, t, ph, pe, step_off);
    return;
  }
  const int2 u = make_int2(t.x & ((1 << KIND_SHIFT) - 1), t.y);
  switch (t.x >> KIND_SHIFT) {
    case KIND_X: tb_tile_nw<T, RPT, K, KIND_X, NW>(a, dst, u, ph, pe, step_off); break;
    case KIND_Y: tb_tile_nw<T, RPT, K, KIND_Y, NW>(a, dst, u, ph, pe, step_off); break;
    default: tb_tile_nw<T, RPT, K, KIND_XY, NW>(a, dst, u, ph, pe, step_off); break;
  }
}

// A column segment of interior tiles in one CTA: an ordinary lean tile (the head, output rows
// [r, r + ER - 2K)) followed by n_carried carried tiles of ER - K output rows each, every one
// taking the row above it from its predecessor (TBCarry). With ER = 5K, a head and three
// carried tiles cover the rows of five ordinary tiles with four tiles' arithmetic.
template <typename T, int RPT, int K, int NW, bool TMM = false>
__global__ void __launch_bounds__(32 * NW, TBShape<T, RPT, K, KIND_INNER, NW>::MIN_BLOCKS)
k_tb_seg(const __grid_constant__ SimArgs<T> a, const __grid_constant__ TBDst<T> dst,
         const int2* __restrict__ segs, int n_carried, const __grid_constant__ PhasePlan<T> ph,
         const __grid_constant__ PhasePlan<T> pe, int step_off) {
  using S = TBShape<T, RPT, K, KIND_INNER, NW>;
  const int2 g = segs[blockIdx.x];
  int r = g.x;
  for (int u = 0; u <= n_carried; ++u) {
    TBCarry<T> c;
    c.par = u & 1;
    c.carried = u > 0;
    tb_tile<T, RPT, K, KIND_INNER, false, TBNoHook, NW, false, TMM, true>(a, dst, make_int2(r, g.y), ph, pe,
                                                                            step_off, nullptr, nullptr, nullptr,
                                                                            TBNoHook(), c);
    r += u == 0 ? S::OR : S::ER - K;
  }
}

// One CPML kind per kernel: each kernel then holds one tile body, which keeps the code of a
// launch within the instruction cache (the three bodies in one kernel did not fit). As for the
// interior tiles, the CPML tiles without a source, monitor or trace node take the lean body
// (PLAN false): fewer registers, and the step is 13 % shorter at 2024² fp32.
template <typename T, int RPT, int K, int KIND, int NW = 8, bool PLAN = true, bool TMM = false>
__global__ void __launch_bounds__(32 * NW, 1)
k_tb_kind(const __grid_constant__ SimArgs<T> a, const __grid_constant__ TBDst<T> dst,
          const int2* __restrict__ tiles, const __grid_constant__ PhasePlan<T> ph,
          const __grid_constant__ PhasePlan<T> pe, int step_off) {
  const int2 t = tiles[blockIdx.x];
  tb_tile_nw<T, RPT, K, KIND, NW, PLAN, TMM>(a, dst, make_int2(t.x & ((1 << KIND_SHIFT) - 1), t.y), ph, pe,
                                             step_off);
}

template <typename T, int RPT, int K, int KIND, int NW = 8, bool PLAN = true>
__global__ void __launch_bounds__(32 * NW, 1)
k_tb_batch_kind(const BatchSim<T>* __restrict__ sims, const int4* __restrict__ tiles, int parity, int step_off) {
  const int4 t = tiles[blockIdx.x];  // simulation, r0, c0, kind
  const BatchSim<T>& b = sims[t.x];
  tb_tile_nw<T, RPT, K, KIND, NW, PLAN>(b.src[parity], b.dst[parity], make_int2(t.y, t.z), b.ph, b.pe, step_off);
}

// Batched form: every tile names its simulation (and, for CPML tiles, its kind in .w); all
// simulations advance the same K steps.
template <typename T, int RPT, int K, bool PML, int NW = 8, bool PLAN = true>
__global__ void __launch_bounds__(32 * NW, TBShape<T, RPT, K, PML ? KIND_XY : KIND_INNER, NW>::MIN_BLOCKS)
k_tb_batch(const BatchSim<T>* __restrict__ sims, const int4* __restrict__ tiles, int parity, int step_off) {
  const int4 t = tiles[blockIdx.x];  // simulation, r0, c0, kind
  const BatchSim<T>& b = sims[t.x];
  const int2 u = make_int2(t.y, t.z);
  if (!PML) {
    tb_tile_nw<T, RPT, K, KIND_INNER, NW, PLAN>(b.src[parity], b.dst[parity], u, b.ph, b.pe, step_off);
    return;
  }
  switch (t.w) {
    case KIND_X: tb_tile_nw<T, RPT, K, KIND_X, NW>(b.src[parity], b.dst[parity], u, b.ph, b.pe, step_off); break;
    case KIND_Y: tb_tile_nw<T, RPT, K, KIND_Y, NW>(b.src[parity], b.dst[parity], u, b.ph, b.pe, step_off); break;
    default: tb_tile_nw<T, RPT, K, KIND_XY, NW>(b.src[parity], b.dst[parity], u, b.ph, b.pe, step_off); break;
  }
}

// Compiled shapes (rows = 8 * RPT, depth K); the CPML variant's six planes must fit 227 KB.
// X(dtype, rows per warp, depth, warps)
// (CPML tiles always run 8 warps on the same tile: rows per warp NW * RPT / 8)
#define ETG_TB_SHAPES_F32(X) \
  X(ETG_F32, 5, 4, 8) X(ETG_F32, 6, 4, 8) X(ETG_F32, 8, 4, 8) X(ETG_F32, 3, 4, 16) X(ETG_F32, 5, 8, 8)
#define ETG_TB_SHAPES_F64(X) X(ETG_F64, 4, 2, 8) X(ETG_F64, 5, 2, 8) X(ETG_F64, 4, 4, 8)

}  // namespace etg
