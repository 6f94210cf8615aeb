// 3D Yee engine: six field components, CPML on PEC faces, periodic axes, point sources and
// DFT monitors, resident in HBM and stepped by CUDA kernels.
//
// Etalon itself stops at 2D TE (etalon/fdtd/capabilities.py:7-24 refuses 3D); this engine
// carries its discretisation to three axes (the layout of etalon/grid/yee.py:27-79 with one
// more axis, the update order of etalon/fdtd/backends/numpy_backend.py:41-61 per component,
// the step order of etalon/fdtd/solver.py:83-128) so that a run invariant along a one-cell
// periodic axis is, bit for bit, the 2D TE run of the other two.
//
// Layout: every array (six fields, twelve psi, three cb) is an (nx+1) x (ny+1) x Pz block
// with Pz = nz + 1 rounded up to 8 elements and z contiguous; component (i, j, k) sits at
// i * (ny+1) * Pz + j * Pz + k whatever its own extent, so one index and one set of strides
// serve all of them. Positions past a component's extent stay zero and are never read.
// psi is stored only for axes that carry CPML, and read or written only inside the strips
// where the profile is not b = 1, c = 0 (psi is exactly +0 everywhere else).
//
// One step is two stencil kernels (H, then E: one thread per (i, j, k), z across the lanes of
// a warp), each followed by its phase's source injection (one thread, NumPy's gather-subtract-
// scatter per source) and DFT accumulation (one thread per frequency and node). Steps run in
// CUDA graphs of up to 32 steps; a device step counter gives every kernel its step n. A fused
// step (one kernel for H and E over two buffer sets, below) is an option with the same bits.
#include <cstring>
#include <map>
#include <vector>

#include "etg_common.cuh"

namespace etg {
namespace {

constexpr int Y3_NFIELD = 6, Y3_NPSI = 12, Y3_NCB = 3;
constexpr int Y3_MAX_SRC = 16, Y3_MAX_MON = 24, Y3_MAX_SRC_NODES = 64;
constexpr int Y3_GRAPH_STEPS = 32;
constexpr int ERR_TABLE = 1;

// psi p belongs to field kPsiComp[p] (0..5: ex ey ez hx hy hz) and differentiates along kPsiAxis[p]
constexpr int kPsiComp[Y3_NPSI] = {3, 3, 4, 4, 5, 5, 0, 0, 1, 1, 2, 2};
constexpr int kPsiAxis[Y3_NPSI] = {1, 2, 2, 0, 0, 1, 1, 2, 2, 0, 0, 1};
// half (1) or integer (0) position of each field along x, y, z
constexpr int kHalf[Y3_NFIELD][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}};

template <typename T>
struct Y3Args {
  int n0, n1, n2;        // cells per axis
  int m0, m1, m2;        // integer positions per axis: n + 1 (PEC walls) or n (periodic)
  int p0, p1, p2;        // periodic axes
  int64_t si, sj;        // strides of i and j; k is contiguous
  T *ex, *ey, *ez, *hx, *hy, *hz;
  T* psi[Y3_NPSI];       // nullptr on axes without CPML
  const T *cb_ex, *cb_ey, *cb_ez;
  const T* prof[3][6];   // per axis: b_e c_e ik_e (integer positions), b_h c_h ik_h (half)
  int lo_e[3], hi_e[3], lo_h[3], hi_h[3];  // positions < lo or >= hi carry psi
  T db, inv_dx, inv_dy, inv_dz;
};

template <typename T>
struct Y3Src {
  T* field;
  const int64_t* idx;
  const T* table;  // (rows, nn): the value subtracted at step n is row n - n0
  int64_t n0, rows;
  int nn;
};

template <typename T>
struct Y3SrcPhase {
  int n;
  Y3Src<T> s[Y3_MAX_SRC];
};

template <typename T>
struct Y3Mon {
  T* acc;          // (nf, nn) complex
  const T* field;
  const int64_t* idx;
  const T* table;  // (rows, nf) complex phasors
  int64_t n0, rows;
  int nn, nf;
};

template <typename T>
struct Y3MonPhase {
  int n;
  Y3Mon<T> m[Y3_MAX_MON];
};

// CPML term of an update along `axis` at position `pos` (W = 0: integer positions, E updates;
// W = 1: half positions, H updates): psi <- b psi + c d, then d / kappa + psi
// (numpy_backend.py:41-61 per axis). Outside the strips b = 1, c = 0, 1/kappa = 1 and psi is +0,
// so the term is d + 0 exactly and nothing is loaded. Inside (`strip`, worked out once per axis
// and thread), psi and the profile are read here, after the field loads: strip cells pay the
// extra round trip, the others keep few registers (many cells in flight per SM).
template <typename T, int W>
__device__ __forceinline__ T term(const Y3Args<T>& a, bool strip, int p, int axis, int pos, int64_t idx, T d) {
  if (!strip) return add(d, T(0));
  T* const psi = a.psi[p];
  const T* const* pr = a.prof[axis] + 3 * W;
  const T v = add(mul(pr[0][pos], psi[idx]), mul(pr[1][pos], d));
  psi[idx] = v;
  return add(mul(d, pr[2][pos]), v);
}

// whether position `pos` along `axis` lies in a CPML strip of the H (W = 1) or E (W = 0) profile
template <typename T, int W>
__device__ __forceinline__ bool in_strip(const Y3Args<T>& a, int axis, int pos) {
  const int lo = W ? a.lo_h[axis] : a.lo_e[axis], hi = W ? a.hi_h[axis] : a.hi_e[axis];
  return a.psi[axis == 0 ? 3 : axis == 1 ? 0 : 1] != nullptr && (pos < lo || pos >= hi);
}

// H^(n-1/2) -> H^(n+1/2) from E^n: forward differences (PER: the +1 neighbour wraps to 0 on a
// periodic axis). Hx lives at (integer x, half y, half z), Hy at (half, integer, half), Hz at
// (half, half, integer). One thread per (i, j, k), z across the lanes of a warp; all field
// loads first, then the three updates.
template <typename T, bool PER>
__global__ void __launch_bounds__(256) k3_update_h(const Y3Args<T> a) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= a.m2 || j >= a.m1) return;
  const int64_t idx = i * a.si + j * a.sj + k;
  const int dk = (PER && a.p2 && k + 1 == a.n2) ? -k : 1;
  const int dj = (PER && a.p1 && j + 1 == a.n1) ? -j * (int)a.sj : (int)a.sj;
  const int64_t di = (PER && a.p0 && i + 1 == a.n0) ? -(int64_t)i * a.si : a.si;
  const bool vx = j < a.n1 && k < a.n2, vy = i < a.n0 && k < a.n2, vz = i < a.n0 && j < a.n1;
  const T* __restrict__ ex = a.ex + idx;
  const T* __restrict__ ey = a.ey + idx;
  const T* __restrict__ ez = a.ez + idx;
  const T ex0 = ex[0], ey0 = ey[0], ez0 = ez[0];  // every (i, j, k) of the block is in the arrays
  const T hx0 = a.hx[idx], hy0 = a.hy[idx], hz0 = a.hz[idx];
  const T ey_k = vx ? ey[dk] : T(0), ez_j = vx ? ez[dj] : T(0);
  const T ez_i = vy ? ez[di] : T(0), ex_k = vy ? ex[dk] : T(0);
  const T ex_j = vz ? ex[dj] : T(0), ey_i = vz ? ey[di] : T(0);
  // (the strip tests are evaluated where they are used: held across the loads they cost the
  // fp32 kernel registers and occupancy)
  if (vx) {
    const T tz = term<T, 1>(a, in_strip<T, 1>(a, 2, k), 1, 2, k, idx, mul(sub(ey_k, ey0), a.inv_dz));
    const T ty = term<T, 1>(a, in_strip<T, 1>(a, 1, j), 0, 1, j, idx, mul(sub(ez_j, ez0), a.inv_dy));
    a.hx[idx] = add(hx0, mul(a.db, sub(tz, ty)));
  }
  if (vy) {
    const T tx = term<T, 1>(a, in_strip<T, 1>(a, 0, i), 3, 0, i, idx, mul(sub(ez_i, ez0), a.inv_dx));
    const T tz = term<T, 1>(a, in_strip<T, 1>(a, 2, k), 2, 2, k, idx, mul(sub(ex_k, ex0), a.inv_dz));
    a.hy[idx] = add(hy0, mul(a.db, sub(tx, tz)));
  }
  if (vz) {
    const T ty = term<T, 1>(a, in_strip<T, 1>(a, 1, j), 5, 1, j, idx, mul(sub(ex_j, ex0), a.inv_dy));
    const T tx = term<T, 1>(a, in_strip<T, 1>(a, 0, i), 4, 0, i, idx, mul(sub(ey_i, ey0), a.inv_dx));
    a.hz[idx] = add(hz0, mul(a.db, sub(ty, tx)));
  }
}

// E^n -> E^(n+1) from H^(n+1/2): backward differences at the integer positions off the PEC
// walls (1 .. n-1), or at all n on a periodic axis (PER; the -1 neighbour of 0 is n-1).
// Tangential E on a wall is never written and stays as it is. All loads first, then the
// three updates.
template <typename T, bool PER>
__global__ void __launch_bounds__(256) k3_update_e(const Y3Args<T> a) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= a.m2 || j >= a.m1) return;
  const int64_t idx = i * a.si + j * a.sj + k;
  const bool in_i = (PER && a.p0) ? i < a.n0 : (i >= 1 && i < a.n0);
  const bool in_j = (PER && a.p1) ? j < a.n1 : (j >= 1 && j < a.n1);
  const bool in_k = (PER && a.p2) ? k < a.n2 : (k >= 1 && k < a.n2);
  const int bk = (PER && k == 0) ? a.n2 - 1 : -1;
  const int bj = (PER && j == 0) ? (a.n1 - 1) * (int)a.sj : -(int)a.sj;
  const int64_t bi = (PER && i == 0) ? (int64_t)(a.n0 - 1) * a.si : -a.si;
  const bool vx = i < a.n0 && in_j && in_k, vy = in_i && j < a.n1 && in_k, vz = in_i && in_j && k < a.n2;
  const T* __restrict__ hx = a.hx + idx;
  const T* __restrict__ hy = a.hy + idx;
  const T* __restrict__ hz = a.hz + idx;
  const T hx0 = hx[0], hy0 = hy[0], hz0 = hz[0];
  const T hz_j = vx ? hz[bj] : T(0), hy_k = vx ? hy[bk] : T(0);
  const T hz_i = vy ? hz[bi] : T(0), hx_k = vy ? hx[bk] : T(0);
  const T hy_i = vz ? hy[bi] : T(0), hx_j = vz ? hx[bj] : T(0);
  const T ex0 = vx ? a.ex[idx] : T(0), cx = vx ? a.cb_ex[idx] : T(0);
  const T ey0 = vy ? a.ey[idx] : T(0), cy = vy ? a.cb_ey[idx] : T(0);
  const T ez0 = vz ? a.ez[idx] : T(0), cz = vz ? a.cb_ez[idx] : T(0);
  const bool sx = in_strip<T, 0>(a, 0, i), sy = in_strip<T, 0>(a, 1, j), sz = in_strip<T, 0>(a, 2, k);
  if (vx) {
    const T ty = term<T, 0>(a, sy, 6, 1, j, idx, mul(sub(hz0, hz_j), a.inv_dy));
    const T tz = term<T, 0>(a, sz, 7, 2, k, idx, mul(sub(hy0, hy_k), a.inv_dz));
    a.ex[idx] = add(ex0, mul(cx, sub(ty, tz)));
  }
  if (vy) {
    const T tx = term<T, 0>(a, sx, 9, 0, i, idx, mul(sub(hz0, hz_i), a.inv_dx));
    const T tz = term<T, 0>(a, sz, 8, 2, k, idx, mul(sub(hx0, hx_k), a.inv_dz));
    a.ey[idx] = sub(ey0, mul(cy, sub(tx, tz)));
  }
  if (vz) {
    const T tx = term<T, 0>(a, sx, 10, 0, i, idx, mul(sub(hy0, hy_i), a.inv_dx));
    const T ty = term<T, 0>(a, sy, 11, 1, j, idx, mul(sub(hx0, hx_j), a.inv_dy));
    a.ez[idx] = add(ez0, mul(cz, sub(tx, ty)));
  }
}

// field[nodes] -= delta, source by source, each as NumPy does it: gather every node, subtract,
// then scatter (a node listed twice keeps its last value). A handful of nodes: one thread.
template <typename T>
__global__ void k3_inject(const Y3SrcPhase<T> p, const int64_t* step, int s_off, int* flag) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t n = *step + s_off;
  for (int q = 0; q < p.n; ++q) {
    const Y3Src<T>& s = p.s[q];
    const int64_t r = n - s.n0;
    if (r < 0 || r >= s.rows) {
      atomicOr(flag, ERR_TABLE);
      continue;
    }
    T vals[Y3_MAX_SRC_NODES];
    for (int m = 0; m < s.nn; ++m) vals[m] = sub(s.field[s.idx[m]], s.table[r * s.nn + m]);
    for (int m = 0; m < s.nn; ++m) s.field[s.idx[m]] = vals[m];
  }
}

// acc[f, node] += field[node] * phasor[f] for every monitor of a phase (blockIdx.y): the
// value (v + 0i)(re + i im) = (v re, v im), then a complex add (numpy_backend.py:63-67).
template <typename T>
__global__ void k3_dft(const Y3MonPhase<T> p, const int64_t* step, int s_off, int* flag) {
  const Y3Mon<T>& m = p.m[blockIdx.y];
  const int64_t n = *step + s_off;
  const int64_t r = n - m.n0;
  if (r < 0 || r >= m.rows) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(flag, ERR_TABLE);
    return;
  }
  const int pairs = m.nn * m.nf;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < pairs; q += gridDim.x * blockDim.x) {
    const int f = q / m.nn, node = q - f * m.nn;
    const T v = m.field[m.idx[node]];
    const T* ph = m.table + 2 * (r * m.nf + f);
    const int64_t o = 2 * ((int64_t)f * m.nn + node);
    m.acc[o] = add(m.acc[o], mul(v, ph[0]));
    m.acc[o + 1] = add(m.acc[o + 1], mul(v, ph[1]));
  }
}

// ---------------------------------------------------------------------------- fused step
// One kernel per step, H and E together, from one buffer set (src) into the other (dst): a
// step reads E, H and cb once and writes E and H once (60 B per cell in fp32, against 84 for
// the two kernels). A block covers 7 rows (y) x 31 columns (z) of owned cells plus one halo
// row and column below them, and walks a chunk of x planes: at plane i every thread computes
// H(i) at its position (halo threads included, on the wrapped position along a periodic axis)
// from src; rows exchange Hz and Hx through shared memory, columns Hy and Hx by shuffle, Hz and
// Hy of plane i - 1 stay in registers, and the owning threads then update E(i). Every H
// position is owned by one block, which writes it; a block's halo and the plane before its
// chunk are recomputed, not written. psi comes from src and goes to dst the same way. Point
// sources are applied where their node is computed (H sources by every thread that computes
// the node, halo included, before E reads it; E sources after the E update), each source as
// NumPy's gather-subtract-scatter does it (a node listed twice keeps its last delta).
// Positions no update writes (tangential E on a PEC wall) are equal in both sets.
// Measured at 524 x 524 x 174 fp32 it is the slower form: 1.52 ms per step against 0.88 ms
// for the two kernels. DRAM moves 78 B per cell (the halo row and column and the plane before
// each chunk are read again), the halo recompute adds instructions, and the barrier per plane
// stalls 8 warps at 5 CTAs per SM (16-row blocks: 1.81 ms). It stays an option, not the default.
constexpr int Y3F_NODES = 32, Y3F_SRC = 16, Y3F_CH = 16, Y3F_ROWS = 8;

struct Y3FNode {
  int i, j, k;
  int8_t comp, slot;
  int16_t col;
};

template <typename T>
struct Y3FSrc {
  int n;                    // nodes, in the order their deltas are subtracted
  Y3FNode node[Y3F_NODES];
  const T* tab[Y3F_SRC];    // (rows, nn) per source
  int64_t n0[Y3F_SRC], rows[Y3F_SRC];
  int nn[Y3F_SRC];
};

template <typename T>
struct Y3Fused {
  Y3Args<T> a;                         // src fields and psi, coefficients
  T *dex, *dey, *dez, *dhx, *dhy, *dhz;  // dst fields
  T* dpsi[Y3_NPSI];                    // dst psi
  Y3FSrc<T> hs, es;
  const int64_t* step;
  int s_off;
  int* flag;
};

// CPML term from src psi; the new psi goes to dst when `keep`.
template <typename T, int W>
__device__ __forceinline__ T term2(const Y3Args<T>& a, T* const* dpsi, int p, int axis, int pos, int64_t idx, T d,
                                   bool keep) {
  const T* psi = a.psi[p];
  const int lo = W ? a.lo_h[axis] : a.lo_e[axis], hi = W ? a.hi_h[axis] : a.hi_e[axis];
  if (psi == nullptr || (pos >= lo && pos < hi)) return add(d, T(0));
  const T* const* pr = a.prof[axis] + 3 * W;
  const T v = add(mul(pr[0][pos], psi[idx]), mul(pr[1][pos], d));
  if (keep) dpsi[p][idx] = v;
  return add(mul(d, pr[2][pos]), v);
}

// subtract the deltas of the sources whose node is (i, j, k) of component c (mask: this
// thread's candidate nodes)
template <typename T>
__device__ __forceinline__ T inject(const Y3FSrc<T>& q, uint32_t mask, int i, int c, int64_t n, T v, int* flag) {
  for (; mask; mask &= mask - 1) {
    const Y3FNode& d = q.node[__ffs(mask) - 1];
    if (d.i != i || d.comp != c) continue;
    const int64_t r = n - q.n0[d.slot];
    if (r < 0 || r >= q.rows[d.slot]) {
      atomicOr(flag, ERR_TABLE);
      continue;
    }
    v = sub(v, q.tab[d.slot][r * q.nn[d.slot] + d.col]);
  }
  return v;
}

template <typename T>
__global__ void __launch_bounds__(32 * Y3F_ROWS) k3_step_fused(const Y3Fused<T> P) {
  const Y3Args<T>& a = P.a;
  __shared__ T sHz[2][Y3F_ROWS][32], sHx[2][Y3F_ROWS][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int k = blockIdx.x * 31 - 1 + tx, j = blockIdx.y * (Y3F_ROWS - 1) - 1 + ty;
  const int ib = blockIdx.z * Y3F_CH, ie = min(ib + Y3F_CH, a.m0);
  // the position this thread computes H at (wrapped on a periodic axis; -1: none)
  const int kw = k < 0 ? (a.p2 ? k + a.n2 : -1) : (k < a.m2 ? k : -1);
  const int jw = j < 0 ? (a.p1 ? j + a.n1 : -1) : (j < a.m1 ? j : -1);
  const bool live = kw >= 0 && jw >= 0;
  const bool own = live && tx >= 1 && ty >= 1;
  const int64_t n = *P.step + P.s_off;
  uint32_t hmask = 0, emask = 0;
  for (int q = 0; q < P.hs.n; ++q)
    if (P.hs.node[q].j == jw && P.hs.node[q].k == kw) hmask |= 1u << q;
  if (own)
    for (int q = 0; q < P.es.n; ++q)
      if (P.es.node[q].j == jw && P.es.node[q].k == kw) emask |= 1u << q;
  const int dk = (a.p2 && kw + 1 == a.n2) ? -kw : 1;
  const int dj = (a.p1 && jw + 1 == a.n1) ? -jw * (int)a.sj : (int)a.sj;
  const int64_t jk = (int64_t)jw * a.sj + kw;
  const bool in_j = a.p1 ? jw < a.n1 : (jw >= 1 && jw < a.n1);
  const bool in_k = a.p2 ? kw < a.n2 : (kw >= 1 && kw < a.n2);
  T hz_p = T(0), hy_p = T(0);
  int par = 0;
  for (int i = ib - 1; i < ie; ++i, par ^= 1) {
    const bool warm = i < ib;  // the plane before the chunk: H only, not written
    const int iw = i < 0 ? (a.p0 ? i + a.n0 : -1) : i;
    T hx_c = T(0), hy_c = T(0), hz_c = T(0), ex0 = T(0), ey0 = T(0), ez0 = T(0);
    if (live && iw >= 0) {
      const int64_t idx = iw * a.si + jk;
      const int64_t di = (a.p0 && iw + 1 == a.n0) ? -(int64_t)iw * a.si : a.si;
      const bool vx = jw < a.n1 && kw < a.n2, vy = iw < a.n0 && kw < a.n2, vz = iw < a.n0 && jw < a.n1;
      const T* __restrict__ ex = a.ex + idx;
      const T* __restrict__ ey = a.ey + idx;
      const T* __restrict__ ez = a.ez + idx;
      ex0 = ex[0], ey0 = ey[0], ez0 = ez[0];
      const T hx0 = a.hx[idx], hy0 = a.hy[idx], hz0 = a.hz[idx];
      const T ey_k = vx ? ey[dk] : T(0), ez_j = vx ? ez[dj] : T(0);
      const T ez_i = vy ? ez[di] : T(0), ex_k = vy ? ex[dk] : T(0);
      const T ex_j = vz ? ex[dj] : T(0), ey_i = vz ? ey[di] : T(0);
      const bool keep = own && !warm;
      if (vx) {
        const T tz = term2<T, 1>(a, P.dpsi, 1, 2, kw, idx, mul(sub(ey_k, ey0), a.inv_dz), keep);
        const T ty_ = term2<T, 1>(a, P.dpsi, 0, 1, jw, idx, mul(sub(ez_j, ez0), a.inv_dy), keep);
        hx_c = inject(P.hs, hmask, iw, 3, n, add(hx0, mul(a.db, sub(tz, ty_))), P.flag);
        if (keep) P.dhx[idx] = hx_c;
      }
      if (vy) {
        const T tx_ = term2<T, 1>(a, P.dpsi, 3, 0, iw, idx, mul(sub(ez_i, ez0), a.inv_dx), keep);
        const T tz = term2<T, 1>(a, P.dpsi, 2, 2, kw, idx, mul(sub(ex_k, ex0), a.inv_dz), keep);
        hy_c = inject(P.hs, hmask, iw, 4, n, add(hy0, mul(a.db, sub(tx_, tz))), P.flag);
        if (keep) P.dhy[idx] = hy_c;
      }
      if (vz) {
        const T ty_ = term2<T, 1>(a, P.dpsi, 5, 1, jw, idx, mul(sub(ex_j, ex0), a.inv_dy), keep);
        const T tx_ = term2<T, 1>(a, P.dpsi, 4, 0, iw, idx, mul(sub(ey_i, ey0), a.inv_dx), keep);
        hz_c = inject(P.hs, hmask, iw, 5, n, add(hz0, mul(a.db, sub(ty_, tx_))), P.flag);
        if (keep) P.dhz[idx] = hz_c;
      }
    }
    sHz[par][ty][tx] = hz_c;
    sHx[par][ty][tx] = hx_c;
    const T hy_km = __shfl_up_sync(0xffffffffu, hy_c, 1), hx_km = __shfl_up_sync(0xffffffffu, hx_c, 1);
    __syncthreads();
    if (!warm && own) {
      const int64_t idx = (int64_t)i * a.si + jk;
      const bool in_i = a.p0 ? i < a.n0 : (i >= 1 && i < a.n0);
      const T hz_jm = sHz[par][ty - 1][tx], hx_jm = sHx[par][ty - 1][tx];
      if (i < a.n0 && in_j && in_k) {
        const T ty_ = term2<T, 0>(a, P.dpsi, 6, 1, jw, idx, mul(sub(hz_c, hz_jm), a.inv_dy), true);
        const T tz = term2<T, 0>(a, P.dpsi, 7, 2, kw, idx, mul(sub(hy_c, hy_km), a.inv_dz), true);
        P.dex[idx] = inject(P.es, emask, i, 0, n, add(ex0, mul(a.cb_ex[idx], sub(ty_, tz))), P.flag);
      }
      if (in_i && jw < a.n1 && in_k) {
        const T tx_ = term2<T, 0>(a, P.dpsi, 9, 0, i, idx, mul(sub(hz_c, hz_p), a.inv_dx), true);
        const T tz = term2<T, 0>(a, P.dpsi, 8, 2, kw, idx, mul(sub(hx_c, hx_km), a.inv_dz), true);
        P.dey[idx] = inject(P.es, emask, i, 1, n, sub(ey0, mul(a.cb_ey[idx], sub(tx_, tz))), P.flag);
      }
      if (in_i && in_j && kw < a.n2) {
        const T tx_ = term2<T, 0>(a, P.dpsi, 10, 0, i, idx, mul(sub(hy_c, hy_p), a.inv_dx), true);
        const T ty_ = term2<T, 0>(a, P.dpsi, 11, 1, jw, idx, mul(sub(hx_c, hx_jm), a.inv_dy), true);
        P.dez[idx] = inject(P.es, emask, i, 2, n, add(ez0, mul(a.cb_ez[idx], sub(tx_, ty_))), P.flag);
      }
    }
    hz_p = hz_c, hy_p = hy_c;
  }
}

__global__ void k3_step_add(int64_t* step, int g) { *step += g; }

}  // namespace
}  // namespace etg

using namespace etg;

struct etg_yee3d {
  int dtype = ETG_F32;
  int n[3] = {}, m[3] = {}, per[3] = {};
  int64_t pz = 0, sj = 0, si = 0;
  size_t elems = 0;
  // two sets of fields and psi: the state is in set `cur`; the fused step writes the other
  // set and flips `cur` (set 1 is allocated at the first fused step)
  void* f[2][Y3_NFIELD] = {};
  void* psi[2][Y3_NPSI] = {};
  int cur = 0;
  bool two_sets = false;
  bool fused = false;  // ETG3_OPT_FUSED
  void* cb[Y3_NCB] = {};
  void* prof[3][6] = {};
  int lo_e[3] = {}, hi_e[3] = {}, lo_h[3] = {}, hi_h[3] = {};
  double scal[4] = {};  // db, 1/dx, 1/dy, 1/dz (values of the run's dtype)
  bool have_scal = false;
  struct Src {
    int comp, nn;
    int64_t* idx;
    void* table;
    int64_t n0, rows;
    std::vector<int64_t> host_idx;  // the padded node indices, for the fused step's node list
  };
  struct Mon {
    int comp, nn, nf;
    int64_t* idx;
    void* acc;
    void* table;
    int64_t n0, rows;
  };
  std::vector<Src> src;
  std::vector<Mon> mon;
  int64_t* d_step = nullptr;
  int* d_flag = nullptr;
  int64_t h_step = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0;
  int64_t last_launches = 0;
  std::map<int, cudaGraphExec_t> graphs;  // keyed by the starting set (+2 for the fused step)
  std::map<int, int64_t> graph_launches;
};

namespace {

size_t esize(const etg_yee3d* s) { return s->dtype == ETG_F32 ? 4 : 8; }

// cudaMalloc that leaves *p null when it fails (so a later attempt or destroy sees no array)
bool dev_alloc(void** p, size_t bytes) {
  if (cudaMalloc(p, bytes) == cudaSuccess) return true;
  *p = nullptr;
  (void)cudaGetLastError();
  return false;
}

// extent of field c (0..5) along each axis
void extent(const etg_yee3d* s, int c, int64_t out[3]) {
  for (int a = 0; a < 3; ++a) out[a] = kHalf[c][a] ? s->n[a] : s->m[a];
}

void drop_graphs(etg_yee3d* s) {
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
  s->graph_launches.clear();
}

template <typename T>
Y3Args<T> args_of(const etg_yee3d* s, int set) {
  Y3Args<T> a{};
  a.n0 = s->n[0], a.n1 = s->n[1], a.n2 = s->n[2];
  a.m0 = s->m[0], a.m1 = s->m[1], a.m2 = s->m[2];
  a.p0 = s->per[0], a.p1 = s->per[1], a.p2 = s->per[2];
  a.si = s->si, a.sj = s->sj;
  T* const* f = reinterpret_cast<T* const*>(s->f[set]);
  a.ex = f[0], a.ey = f[1], a.ez = f[2], a.hx = f[3], a.hy = f[4], a.hz = f[5];
  for (int p = 0; p < Y3_NPSI; ++p) a.psi[p] = static_cast<T*>(s->psi[set][p]);
  a.cb_ex = static_cast<const T*>(s->cb[0]);
  a.cb_ey = static_cast<const T*>(s->cb[1]);
  a.cb_ez = static_cast<const T*>(s->cb[2]);
  for (int x = 0; x < 3; ++x) {
    for (int q = 0; q < 6; ++q) a.prof[x][q] = static_cast<const T*>(s->prof[x][q]);
    a.lo_e[x] = s->lo_e[x], a.hi_e[x] = s->hi_e[x], a.lo_h[x] = s->lo_h[x], a.hi_h[x] = s->hi_h[x];
  }
  a.db = (T)s->scal[0], a.inv_dx = (T)s->scal[1], a.inv_dy = (T)s->scal[2], a.inv_dz = (T)s->scal[3];
  return a;
}

template <typename T>
void phases_of(const etg_yee3d* s, bool magnetic, int set, Y3SrcPhase<T>* sp, Y3MonPhase<T>* mp) {
  std::memset(sp, 0, sizeof(*sp));
  std::memset(mp, 0, sizeof(*mp));
  for (const auto& q : s->src) {
    if ((q.comp >= 3) != magnetic) continue;
    Y3Src<T>& d = sp->s[sp->n++];
    d.field = static_cast<T*>(s->f[set][q.comp]);
    d.idx = q.idx;
    d.table = static_cast<const T*>(q.table);
    d.n0 = q.n0, d.rows = q.rows, d.nn = q.nn;
  }
  for (const auto& q : s->mon) {
    if ((q.comp >= 3) != magnetic) continue;
    Y3Mon<T>& d = mp->m[mp->n++];
    d.acc = static_cast<T*>(q.acc);
    d.field = static_cast<const T*>(s->f[set][q.comp]);
    d.idx = q.idx;
    d.table = static_cast<const T*>(q.table);
    d.n0 = q.n0, d.rows = q.rows, d.nn = q.nn, d.nf = q.nf;
  }
}

int mon_blocks(const etg_yee3d* s, bool magnetic) {
  int most = 0;
  for (const auto& q : s->mon)
    if ((q.comp >= 3) == magnetic) most = std::max(most, q.nn * q.nf);
  return std::max(1, std::min(1024, (most + 255) / 256));
}

// The sources of one phase as the fused kernel's node list, in subtraction order; false when
// they do not fit it (the two-kernel step then runs).
template <typename T>
bool fused_sources(const etg_yee3d* s, bool magnetic, Y3FSrc<T>* out) {
  std::memset(out, 0, sizeof(*out));
  int slot = 0;
  for (const auto& q : s->src) {
    if ((q.comp >= 3) != magnetic) continue;
    if (slot == Y3F_SRC) return false;
    for (int m = 0; m < q.nn; ++m) {
      bool later = false;  // NumPy's scatter keeps the last delta of a node listed twice
      for (int m2 = m + 1; m2 < q.nn; ++m2) later |= q.host_idx[m2] == q.host_idx[m];
      if (later) continue;
      if (out->n == Y3F_NODES) return false;
      const int64_t x = q.host_idx[m];
      Y3FNode& d = out->node[out->n++];
      d.i = (int)(x / s->si), d.j = (int)((x % s->si) / s->sj), d.k = (int)(x % s->sj);
      d.comp = (int8_t)q.comp, d.slot = (int8_t)slot, d.col = (int16_t)m;
    }
    out->tab[slot] = static_cast<const T*>(q.table);
    out->n0[slot] = q.n0, out->rows[slot] = q.rows, out->nn[slot] = q.nn;
    ++slot;
  }
  return true;
}

// The second set: allocated at the first fused step as a copy of the current one (arrays a
// failed earlier attempt allocated are kept, not allocated again; destroy frees them).
int ensure_two_sets(etg_yee3d* s) {
  if (s->two_sets) return ETG_OK;
  const size_t bytes = s->elems * esize(s);
  const int other = s->cur ^ 1;
  for (int c = 0; c < Y3_NFIELD; ++c) {
    if (!s->f[other][c])
      ETG_REQUIRE(dev_alloc(&s->f[other][c], bytes), ETG_ERR_ALLOC,
                  "etg_yee3d: second field set (%zu bytes per array) could not be allocated", bytes);
    ETG_TRY_CUDA(cudaMemcpyAsync(s->f[other][c], s->f[s->cur][c], bytes, cudaMemcpyDeviceToDevice, s->stream));
  }
  for (int p = 0; p < Y3_NPSI; ++p) {
    if (!s->psi[s->cur][p]) continue;
    if (!s->psi[other][p])
      ETG_REQUIRE(dev_alloc(&s->psi[other][p], bytes), ETG_ERR_ALLOC,
                  "etg_yee3d: second psi set could not be allocated");
    ETG_TRY_CUDA(cudaMemcpyAsync(s->psi[other][p], s->psi[s->cur][p], bytes, cudaMemcpyDeviceToDevice, s->stream));
  }
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  s->two_sets = true;
  return ETG_OK;
}

// one fused step from set `set` into the other; returns the number of launches
template <typename T>
int launch_fused(const etg_yee3d* s, int set, const Y3FSrc<T>& hs, const Y3FSrc<T>& es, int s_off, cudaStream_t st,
                 cudaEvent_t* ev = nullptr) {
  Y3Fused<T> P{};
  P.a = args_of<T>(s, set);
  T* const* d = reinterpret_cast<T* const*>(s->f[set ^ 1]);
  P.dex = d[0], P.dey = d[1], P.dez = d[2], P.dhx = d[3], P.dhy = d[4], P.dhz = d[5];
  for (int p = 0; p < Y3_NPSI; ++p) P.dpsi[p] = static_cast<T*>(s->psi[set ^ 1][p]);
  P.hs = hs, P.es = es, P.step = s->d_step, P.s_off = s_off, P.flag = s->d_flag;
  const dim3 block(32, Y3F_ROWS), grid((s->m[2] + 30) / 31, (s->m[1] + Y3F_ROWS - 2) / (Y3F_ROWS - 1),
                                       (s->m[0] + Y3F_CH - 1) / Y3F_CH);
  if (ev) cudaEventRecord(ev[0], st);
  k3_step_fused<T><<<grid, block, 0, st>>>(P);
  if (ev) cudaEventRecord(ev[1], st);
  Y3SrcPhase<T> sp;
  Y3MonPhase<T> mh, me;
  phases_of<T>(s, true, set ^ 1, &sp, &mh);
  phases_of<T>(s, false, set ^ 1, &sp, &me);
  int launches = 1;
  if (mh.n) k3_dft<T><<<dim3(mon_blocks(s, true), mh.n), 256, 0, st>>>(mh, s->d_step, s_off, s->d_flag), ++launches;
  if (me.n) k3_dft<T><<<dim3(mon_blocks(s, false), me.n), 256, 0, st>>>(me, s->d_step, s_off, s->d_flag), ++launches;
  return launches;
}

// one step (s_off: its offset from the device counter); returns the number of launches
template <typename T>
int launch_step(const etg_yee3d* s, const Y3Args<T>& a, const Y3SrcPhase<T>& sh, const Y3MonPhase<T>& mh,
                const Y3SrcPhase<T>& se, const Y3MonPhase<T>& me, int s_off, cudaStream_t st,
                cudaEvent_t* ev = nullptr) {
  const dim3 block(32, 8), grid((s->m[2] + 31) / 32, (s->m[1] + 7) / 8, s->m[0]);
  int launches = 2;
  if (ev) cudaEventRecord(ev[0], st);
  // the H kernel keeps its run-time periodic tests either way: specialised it takes 36 fp32
  // registers (against 32) and loses more in occupancy than it saves in instructions
  const bool per = s->per[0] || s->per[1] || s->per[2];
  k3_update_h<T, true><<<grid, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[1], st);
  if (sh.n) k3_inject<T><<<1, 32, 0, st>>>(sh, s->d_step, s_off, s->d_flag), ++launches;
  if (mh.n) k3_dft<T><<<dim3(mon_blocks(s, true), mh.n), 256, 0, st>>>(mh, s->d_step, s_off, s->d_flag), ++launches;
  if (ev) cudaEventRecord(ev[2], st);
  if (per) k3_update_e<T, true><<<grid, block, 0, st>>>(a);
  else k3_update_e<T, false><<<grid, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[3], st);
  if (se.n) k3_inject<T><<<1, 32, 0, st>>>(se, s->d_step, s_off, s->d_flag), ++launches;
  if (me.n) k3_dft<T><<<dim3(mon_blocks(s, false), me.n), 256, 0, st>>>(me, s->d_step, s_off, s->d_flag), ++launches;
  return launches;
}

template <typename T>
bool use_fused(const etg_yee3d* s, Y3FSrc<T>* hs, Y3FSrc<T>* es) {
  return s->fused && fused_sources<T>(s, true, hs) && fused_sources<T>(s, false, es);
}

// g steps from set `set` at counter offsets 0 .. g-1, then the counter add; returns the set
// the state ends in (the two-kernel step works in place)
template <typename T>
int steps_from(etg_yee3d* s, bool fused, const Y3FSrc<T>& hs, const Y3FSrc<T>& es, int set, int g,
               int64_t* launches) {
  for (int k = 0; k < g; ++k) {
    if (fused) {
      *launches += launch_fused<T>(s, set, hs, es, k, s->stream);
      set ^= 1;
    } else {
      const Y3Args<T> a = args_of<T>(s, set);
      Y3SrcPhase<T> sh, se;
      Y3MonPhase<T> mh, me;
      phases_of<T>(s, true, set, &sh, &mh);
      phases_of<T>(s, false, set, &se, &me);
      *launches += launch_step<T>(s, a, sh, mh, se, me, k, s->stream);
    }
  }
  k3_step_add<<<1, 1, 0, s->stream>>>(s->d_step, g);
  *launches += 1;
  return set;
}

template <typename T>
int advance(etg_yee3d* s, int64_t steps) {
  Y3FSrc<T> hs, es;
  const bool fused = use_fused<T>(s, &hs, &es);
  if (fused) {
    int r = ensure_two_sets(s);
    if (r) return r;
  }
  int64_t launches = 0;
  ETG_TRY_CUDA(cudaEventRecord(s->ev0, s->stream));
  const int g = Y3_GRAPH_STEPS;  // even: a graph ends in the set it starts from
  int64_t left = steps;
  if (left >= g) {
    const int key = s->cur + (fused ? 2 : 0);
    auto it = s->graphs.find(key);
    int64_t per = 0;
    if (it == s->graphs.end()) {
      cudaGraph_t graph = nullptr;
      ETG_TRY_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      steps_from<T>(s, fused, hs, es, s->cur, g, &per);
      cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
      if (e != cudaSuccess) {
        set_error("etg_yee3d_advance: graph capture failed: %s", cudaGetErrorString(e));
        return ETG_ERR_CUDA;
      }
      cudaGraphExec_t exec = nullptr;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        set_error("etg_yee3d_advance: graph instantiation failed: %s", cudaGetErrorString(e));
        return ETG_ERR_CUDA;
      }
      it = s->graphs.emplace(key, exec).first;
      s->graph_launches[key] = per;
    }
    for (; left >= g; left -= g) {
      ETG_TRY_CUDA(cudaGraphLaunch(it->second, s->stream));
      launches += s->graph_launches[key];
    }
  }
  if (left) s->cur = steps_from<T>(s, fused, hs, es, s->cur, (int)left, &launches);
  ETG_LAUNCH_CHECK();
  ETG_TRY_CUDA(cudaEventRecord(s->ev1, s->stream));
  g_launches += launches;
  s->last_launches = launches;
  s->h_step += steps;
  return ETG_OK;
}

// positions of a profile that carry psi: [0, lo) and [hi, len); the rest must be b = 1, c = 0,
// 1/kappa = 1
template <typename T>
void strips(const T* b, const T* c, const T* ik, int len, int* lo, int* hi) {
  auto trivial = [&](int p) { return b[p] == T(1) && c[p] == T(0) && ik[p] == T(1); };
  int l = 0, h = len;
  while (l < len && !trivial(l)) ++l;
  while (h > l && !trivial(h - 1)) --h;
  for (int p = l; p < h; ++p)
    if (!trivial(p)) {  // not a pair of end strips: psi everywhere
      l = len, h = len;
      break;
    }
  *lo = l, *hi = h;
}

int copy_in(etg_yee3d* s, void* dst, const void* host, int c) {
  int64_t e[3];
  extent(s, c, e);
  const size_t z = esize(s);
  for (int64_t i = 0; i < e[0]; ++i)
    ETG_TRY_CUDA(cudaMemcpy2DAsync(static_cast<char*>(dst) + i * s->si * z, s->sj * z,
                                   static_cast<const char*>(host) + i * e[1] * e[2] * z, e[2] * z, e[2] * z, e[1],
                                   cudaMemcpyHostToDevice, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int copy_out(etg_yee3d* s, void* host, const void* src, int c) {
  int64_t e[3];
  extent(s, c, e);
  const size_t z = esize(s);
  for (int64_t i = 0; i < e[0]; ++i)
    ETG_TRY_CUDA(cudaMemcpy2DAsync(static_cast<char*>(host) + i * e[1] * e[2] * z, e[2] * z,
                                   static_cast<const char*>(src) + i * s->si * z, s->sj * z, e[2] * z, e[1],
                                   cudaMemcpyDeviceToHost, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int field_comp(int id) {  // the field whose extent an array id has
  if (id < Y3_NFIELD) return id;
  if (id < Y3_NFIELD + Y3_NPSI) return kPsiComp[id - Y3_NFIELD];
  return id - Y3_NFIELD - Y3_NPSI;
}

// padded index of a flat C-order index into field c; -1 when out of range
int64_t padded(const etg_yee3d* s, int c, int64_t flat) {
  int64_t e[3];
  extent(s, c, e);
  if (flat < 0 || flat >= e[0] * e[1] * e[2]) return -1;
  const int64_t k = flat % e[2], j = (flat / e[2]) % e[1], i = flat / (e[1] * e[2]);
  return i * s->si + j * s->sj + k;
}

int alloc_psi(etg_yee3d* s, int axis) {
  for (int p = 0; p < Y3_NPSI; ++p) {
    if (kPsiAxis[p] != axis) continue;
    for (int set = 0; set < (s->two_sets ? 2 : 1); ++set) {
      if (s->psi[set][p]) continue;
      ETG_REQUIRE(dev_alloc(&s->psi[set][p], s->elems * esize(s)), ETG_ERR_ALLOC,
                  "etg_yee3d: psi allocation of %zu bytes failed", s->elems * esize(s));
      ETG_TRY_CUDA(cudaMemsetAsync(s->psi[set][p], 0, s->elems * esize(s), s->stream));
    }
  }
  return ETG_OK;
}

// n steps, each stencil launch timed alone (events): the fused step's kernel in ms_h and 0 in
// ms_e, or the H and E kernels of the two-kernel step
template <typename T>
int time_kernels(etg_yee3d* s, int n_steps, double* ms_h, double* ms_e) {
  Y3FSrc<T> hs, es;
  const bool fused = use_fused<T>(s, &hs, &es);
  if (fused) {
    int r = ensure_two_sets(s);
    if (r) return r;
  }
  cudaEvent_t ev[4];
  for (auto& e : ev) ETG_TRY_CUDA(cudaEventCreate(&e));
  double th = 0, te = 0;
  int rc = ETG_OK;
  for (int k = 0; k < n_steps; ++k) {
    if (fused) {
      launch_fused<T>(s, s->cur, hs, es, 0, s->stream, ev);
      s->cur ^= 1;
    } else {
      const Y3Args<T> a = args_of<T>(s, s->cur);
      Y3SrcPhase<T> sh, se;
      Y3MonPhase<T> mh, me;
      phases_of<T>(s, true, s->cur, &sh, &mh);
      phases_of<T>(s, false, s->cur, &se, &me);
      launch_step<T>(s, a, sh, mh, se, me, 0, s->stream, ev);
    }
    k3_step_add<<<1, 1, 0, s->stream>>>(s->d_step, 1);
    if (cudaEventSynchronize(ev[1]) != cudaSuccess || (!fused && cudaEventSynchronize(ev[3]) != cudaSuccess)) {
      set_error("etg_yee3d_kernel_timing: %s", cudaGetErrorString(cudaGetLastError()));
      rc = ETG_ERR_CUDA;
      break;
    }
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    if (!fused) cudaEventElapsedTime(&b, ev[2], ev[3]);
    th += a, te += b;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  if (rc) return rc;
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  s->h_step += n_steps;
  *ms_h = th / n_steps;
  *ms_e = te / n_steps;
  return ETG_OK;
}

}  // namespace


extern "C" {

int etg_yee3d_create(etg_yee3d** out, int dtype, int nx, int ny, int nz, int periodic_mask) {
  ETG_REQUIRE(out && dtype_ok(dtype) && nx > 0 && ny > 0 && nz > 0 && periodic_mask >= 0 && periodic_mask < 8,
              ETG_ERR_ARGUMENT, "etg_yee3d_create: bad arguments (dtype %d, %d x %d x %d, periodic %d)", dtype, nx,
              ny, nz, periodic_mask);
  // grid dimensions: x planes on gridDim.z, rows of 8 (7 in the fused step) on gridDim.y; the
  // kernels take row offsets (j * Pz, up to (ny + 1) * Pz) in 32 bits
  ETG_REQUIRE(nx < 65535 && ny < 458738 && (int64_t)(ny + 1) * (((int64_t)nz + 8) / 8 * 8) < (int64_t(1) << 31) &&
                  (int64_t)(nx + 1) * (ny + 1) * (nz + 8) < (int64_t(1) << 40),
              ETG_ERR_ARGUMENT, "etg_yee3d_create: grid %d x %d x %d too large", nx, ny, nz);
  if (fault_injected("etg_yee3d_create")) return ETG_ERR_INJECTED;
  auto* s = new etg_yee3d();
  s->dtype = dtype;
  const int nn[3] = {nx, ny, nz};
  for (int a = 0; a < 3; ++a) {
    s->n[a] = nn[a];
    s->per[a] = (periodic_mask >> a) & 1;
    s->m[a] = nn[a] + (s->per[a] ? 0 : 1);
  }
  s->pz = ((int64_t)nz + 1 + 7) / 8 * 8;
  s->sj = s->pz;
  s->si = (int64_t)(ny + 1) * s->pz;
  s->elems = (size_t)(nx + 1) * s->si;
  const size_t z = esize(s);
  auto fail = [&](int code) {
    etg_yee3d_destroy(s);
    return code;
  };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
    set_error("etg_yee3d_create: stream or event creation failed");
    return fail(ETG_ERR_CUDA);
  }
  for (int c = 0; c < Y3_NFIELD + Y3_NCB; ++c) {
    void** p = c < Y3_NFIELD ? &s->f[0][c] : &s->cb[c - Y3_NFIELD];
    if (!dev_alloc(p, s->elems * z) || cudaMemsetAsync(*p, 0, s->elems * z, s->stream) != cudaSuccess) {
      set_error("etg_yee3d_create: allocation of %zu bytes failed", s->elems * z);
      return fail(ETG_ERR_ALLOC);
    }
  }
  // unit profiles until etg_yee3d_set_profile: no CPML, no psi
  for (int a = 0; a < 3; ++a) {
    const int len[6] = {s->m[a], s->m[a], s->m[a], s->n[a], s->n[a], s->n[a]};
    for (int q = 0; q < 6; ++q) {
      std::vector<double> one(len[q], q % 3 == 1 ? 0.0 : 1.0);
      std::vector<float> onef(one.begin(), one.end());
      if (!dev_alloc(&s->prof[a][q], len[q] * z) ||
          cudaMemcpy(s->prof[a][q], dtype == ETG_F32 ? (const void*)onef.data() : (const void*)one.data(), len[q] * z,
                     cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("etg_yee3d_create: profile allocation failed");
        return fail(ETG_ERR_ALLOC);
      }
    }
    s->lo_e[a] = 0, s->hi_e[a] = s->m[a], s->lo_h[a] = 0, s->hi_h[a] = s->n[a];
  }
  if (!dev_alloc((void**)&s->d_step, sizeof(int64_t)) || !dev_alloc((void**)&s->d_flag, sizeof(int)) ||
      cudaMemsetAsync(s->d_step, 0, sizeof(int64_t), s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stream) != cudaSuccess) {
    set_error("etg_yee3d_create: counter allocation failed");
    return fail(ETG_ERR_ALLOC);
  }
  *out = s;
  return ETG_OK;
}

int etg_yee3d_destroy(etg_yee3d* s) {
  if (!s) return ETG_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graphs(s);
  for (auto& set : s->f)
    for (void* p : set) cudaFree(p);
  for (auto& set : s->psi)
    for (void* p : set) cudaFree(p);
  for (void* p : s->cb) cudaFree(p);
  for (auto& ax : s->prof)
    for (void* p : ax) cudaFree(p);
  for (auto& q : s->src) cudaFree(q.idx), cudaFree(q.table);
  for (auto& q : s->mon) cudaFree(q.idx), cudaFree(q.acc), cudaFree(q.table);
  cudaFree(s->d_step);
  cudaFree(s->d_flag);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return ETG_OK;
}

int etg_yee3d_set_scalars(etg_yee3d* s, const void* host) {
  ETG_REQUIRE(s && host, ETG_ERR_ARGUMENT, "etg_yee3d_set_scalars: null argument");
  for (int q = 0; q < 4; ++q)
    s->scal[q] = s->dtype == ETG_F32 ? (double)static_cast<const float*>(host)[q] : static_cast<const double*>(host)[q];
  s->have_scal = true;
  drop_graphs(s);
  return ETG_OK;
}

int etg_yee3d_set_profile(etg_yee3d* s, int axis, const void* b_e, const void* c_e, const void* ik_e, const void* b_h,
                          const void* c_h, const void* ik_h) {
  ETG_REQUIRE(s && axis >= 0 && axis < 3 && b_e && c_e && ik_e && b_h && c_h && ik_h, ETG_ERR_ARGUMENT,
              "etg_yee3d_set_profile: bad arguments");
  const void* in[6] = {b_e, c_e, ik_e, b_h, c_h, ik_h};
  const int len[6] = {s->m[axis], s->m[axis], s->m[axis], s->n[axis], s->n[axis], s->n[axis]};
  const size_t z = esize(s);
  for (int q = 0; q < 6; ++q)
    ETG_TRY_CUDA(cudaMemcpyAsync(s->prof[axis][q], in[q], len[q] * z, cudaMemcpyHostToDevice, s->stream));
  if (s->dtype == ETG_F32) {
    using F = const float*;
    strips(static_cast<F>(b_e), static_cast<F>(c_e), static_cast<F>(ik_e), len[0], &s->lo_e[axis], &s->hi_e[axis]);
    strips(static_cast<F>(b_h), static_cast<F>(c_h), static_cast<F>(ik_h), len[3], &s->lo_h[axis], &s->hi_h[axis]);
  } else {
    using D = const double*;
    strips(static_cast<D>(b_e), static_cast<D>(c_e), static_cast<D>(ik_e), len[0], &s->lo_e[axis], &s->hi_e[axis]);
    strips(static_cast<D>(b_h), static_cast<D>(c_h), static_cast<D>(ik_h), len[3], &s->lo_h[axis], &s->hi_h[axis]);
  }
  const bool cpml = s->lo_e[axis] > 0 || s->hi_e[axis] < len[0] || s->lo_h[axis] > 0 || s->hi_h[axis] < len[3];
  if (cpml) {
    int r = alloc_psi(s, axis);
    if (r) return r;
  }
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  drop_graphs(s);
  return ETG_OK;
}

int etg_yee3d_set_field(etg_yee3d* s, int id, const void* host) {
  ETG_REQUIRE(s && host && id >= 0 && id < Y3_NFIELD + Y3_NPSI + Y3_NCB, ETG_ERR_ARGUMENT,
              "etg_yee3d_set_field: bad field id %d", id);
  const int c = field_comp(id);
  // fields and psi go to both sets: positions no update writes then stay equal in both
  auto array_of = [&](int set) -> void* {
    return id < Y3_NFIELD ? s->f[set][id] : id < Y3_NFIELD + Y3_NPSI ? s->psi[set][id - Y3_NFIELD] : s->cb[c];
  };
  void* dst = array_of(s->cur);
  if (!dst) {  // psi of an axis without CPML: identically zero, not stored
    int64_t e[3];
    extent(s, c, e);
    const size_t bytes = (size_t)(e[0] * e[1] * e[2]) * esize(s);
    const unsigned char* h = static_cast<const unsigned char*>(host);
    for (size_t b = 0; b < bytes; ++b)
      ETG_REQUIRE(h[b] == 0, ETG_ERR_STATE,
                  "etg_yee3d_set_field: psi %d belongs to an axis without CPML and must be +0", id);
    return ETG_OK;
  }
  int r = copy_in(s, dst, host, c);
  if (r == ETG_OK && s->two_sets && id < Y3_NFIELD + Y3_NPSI) r = copy_in(s, array_of(s->cur ^ 1), host, c);
  return r;
}

int etg_yee3d_get_field(etg_yee3d* s, int id, void* host) {
  ETG_REQUIRE(s && host && id >= 0 && id < Y3_NFIELD + Y3_NPSI + Y3_NCB, ETG_ERR_ARGUMENT,
              "etg_yee3d_get_field: bad field id %d", id);
  const int c = field_comp(id);
  const void* src = id < Y3_NFIELD              ? s->f[s->cur][id]
                    : id < Y3_NFIELD + Y3_NPSI ? s->psi[s->cur][id - Y3_NFIELD]
                                               : s->cb[c];
  if (!src) {
    int64_t e[3];
    extent(s, c, e);
    std::memset(host, 0, (size_t)(e[0] * e[1] * e[2]) * esize(s));
    return ETG_OK;
  }
  return copy_out(s, host, src, c);
}

int etg_yee3d_add_source(etg_yee3d* s, int component, int n_nodes, const int64_t* flat, int64_t n0, int64_t rows,
                         const void* table) {
  ETG_REQUIRE(s && flat && table && component >= 0 && component < Y3_NFIELD && n_nodes > 0 &&
                  n_nodes <= Y3_MAX_SRC_NODES && rows > 0 && n0 >= 0,
              ETG_ERR_ARGUMENT, "etg_yee3d_add_source: bad arguments (component %d, %d nodes, %lld rows)", component,
              n_nodes, (long long)rows);
  int in_phase = 0;
  for (const auto& q : s->src) in_phase += (q.comp >= 3) == (component >= 3);
  ETG_REQUIRE(in_phase < Y3_MAX_SRC, ETG_ERR_ARGUMENT, "etg_yee3d_add_source: at most %d sources per phase",
              Y3_MAX_SRC);
  std::vector<int64_t> idx(n_nodes);
  for (int k = 0; k < n_nodes; ++k) {
    idx[k] = padded(s, component, flat[k]);
    ETG_REQUIRE(idx[k] >= 0, ETG_ERR_ARGUMENT, "etg_yee3d_add_source: node %lld outside component %d",
                (long long)flat[k], component);
  }
  etg_yee3d::Src q{component, n_nodes, nullptr, nullptr, n0, rows, idx};
  const size_t tb = (size_t)rows * n_nodes * esize(s);
  if (!dev_alloc((void**)&q.idx, n_nodes * sizeof(int64_t)) || !dev_alloc(&q.table, tb)) {
    cudaFree(q.idx);
    set_error("etg_yee3d_add_source: allocation failed");
    return ETG_ERR_ALLOC;
  }
  s->src.push_back(q);
  ETG_TRY_CUDA(cudaMemcpy(q.idx, idx.data(), n_nodes * sizeof(int64_t), cudaMemcpyHostToDevice));
  ETG_TRY_CUDA(cudaMemcpy(q.table, table, tb, cudaMemcpyHostToDevice));
  drop_graphs(s);
  return ETG_OK;
}

int etg_yee3d_add_monitor(etg_yee3d* s, int component, int n_nodes, const int64_t* flat, int n_f, int64_t n0,
                          int64_t rows, const void* table) {
  ETG_REQUIRE(s && flat && table && component >= 0 && component < Y3_NFIELD && n_nodes > 0 && n_f > 0 && rows > 0 &&
                  n0 >= 0 && (int64_t)n_nodes * n_f < (int64_t(1) << 31),
              ETG_ERR_ARGUMENT, "etg_yee3d_add_monitor: bad arguments");
  int in_phase = 0;
  for (const auto& q : s->mon) in_phase += (q.comp >= 3) == (component >= 3);
  ETG_REQUIRE(in_phase < Y3_MAX_MON, ETG_ERR_ARGUMENT, "etg_yee3d_add_monitor: at most %d monitors per phase",
              Y3_MAX_MON);
  std::vector<int64_t> idx(n_nodes);
  for (int k = 0; k < n_nodes; ++k) {
    idx[k] = padded(s, component, flat[k]);
    ETG_REQUIRE(idx[k] >= 0, ETG_ERR_ARGUMENT, "etg_yee3d_add_monitor: node %lld outside component %d",
                (long long)flat[k], component);
  }
  etg_yee3d::Mon q{component, n_nodes, n_f, nullptr, nullptr, nullptr, n0, rows};
  const size_t ab = (size_t)2 * n_nodes * n_f * esize(s), tb = (size_t)2 * rows * n_f * esize(s);
  if (!dev_alloc((void**)&q.idx, n_nodes * sizeof(int64_t)) || !dev_alloc(&q.acc, ab) || !dev_alloc(&q.table, tb)) {
    cudaFree(q.idx);
    cudaFree(q.acc);
    set_error("etg_yee3d_add_monitor: allocation failed");
    return ETG_ERR_ALLOC;
  }
  s->mon.push_back(q);
  ETG_TRY_CUDA(cudaMemcpy(q.idx, idx.data(), n_nodes * sizeof(int64_t), cudaMemcpyHostToDevice));
  ETG_TRY_CUDA(cudaMemset(q.acc, 0, ab));
  ETG_TRY_CUDA(cudaMemcpy(q.table, table, tb, cudaMemcpyHostToDevice));
  drop_graphs(s);
  return ETG_OK;
}

int etg_yee3d_get_dft(etg_yee3d* s, int monitor, void* host) {
  ETG_REQUIRE(s && host && monitor >= 0 && monitor < (int)s->mon.size(), ETG_ERR_ARGUMENT,
              "etg_yee3d_get_dft: bad monitor %d", monitor);
  const auto& q = s->mon[monitor];
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  ETG_TRY_CUDA(cudaMemcpy(host, q.acc, (size_t)2 * q.nn * q.nf * esize(s), cudaMemcpyDeviceToHost));
  return ETG_OK;
}

int etg_yee3d_advance(etg_yee3d* s, int64_t n_steps) {
  ETG_REQUIRE(s && n_steps >= 0, ETG_ERR_ARGUMENT, "etg_yee3d_advance: bad arguments");
  ETG_REQUIRE(s->have_scal, ETG_ERR_STATE, "etg_yee3d_advance: etg_yee3d_set_scalars was not called");
  if (fault_injected("etg_yee3d_advance")) return ETG_ERR_INJECTED;
  for (const auto& q : s->src)
    ETG_REQUIRE(q.n0 <= s->h_step && s->h_step + n_steps <= q.n0 + q.rows, ETG_ERR_STATE,
                "etg_yee3d_advance: a source table covers steps [%lld, %lld), not [%lld, %lld)", (long long)q.n0,
                (long long)(q.n0 + q.rows), (long long)s->h_step, (long long)(s->h_step + n_steps));
  for (const auto& q : s->mon)
    ETG_REQUIRE(q.n0 <= s->h_step && s->h_step + n_steps <= q.n0 + q.rows, ETG_ERR_STATE,
                "etg_yee3d_advance: a phasor table covers steps [%lld, %lld), not [%lld, %lld)", (long long)q.n0,
                (long long)(q.n0 + q.rows), (long long)s->h_step, (long long)(s->h_step + n_steps));
  if (n_steps == 0) return ETG_OK;
  return s->dtype == ETG_F32 ? advance<float>(s, n_steps) : advance<double>(s, n_steps);
}

int etg_yee3d_synchronize(etg_yee3d* s) {
  ETG_REQUIRE(s, ETG_ERR_ARGUMENT, "etg_yee3d_synchronize: null handle");
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  int flag = 0;
  ETG_TRY_CUDA(cudaMemcpy(&flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost));
  ETG_REQUIRE(flag == 0, ETG_ERR_STATE, "etg_yee3d: a source or phasor table did not cover a step (flags %d)", flag);
  return ETG_OK;
}

int etg_yee3d_step_index(etg_yee3d* s, int64_t* n) {
  ETG_REQUIRE(s && n, ETG_ERR_ARGUMENT, "etg_yee3d_step_index: null argument");
  *n = s->h_step;
  return ETG_OK;
}

int etg_yee3d_last_timing(etg_yee3d* s, double* ms, int64_t* launches) {
  ETG_REQUIRE(s && ms && launches, ETG_ERR_ARGUMENT, "etg_yee3d_last_timing: null argument");
  ETG_TRY_CUDA(cudaEventSynchronize(s->ev1));
  float t = 0;
  ETG_TRY_CUDA(cudaEventElapsedTime(&t, s->ev0, s->ev1));
  *ms = t;
  *launches = s->last_launches;
  return ETG_OK;
}

int etg_yee3d_kernel_timing(etg_yee3d* s, int n_steps, double* ms_h, double* ms_e) {
  ETG_REQUIRE(s && ms_h && ms_e && n_steps > 0, ETG_ERR_ARGUMENT, "etg_yee3d_kernel_timing: bad arguments");
  ETG_REQUIRE(s->have_scal, ETG_ERR_STATE, "etg_yee3d_kernel_timing: etg_yee3d_set_scalars was not called");
  for (const auto& q : s->src)
    ETG_REQUIRE(q.n0 <= s->h_step && s->h_step + n_steps <= q.n0 + q.rows, ETG_ERR_STATE,
                "etg_yee3d_kernel_timing: a source table does not cover the steps");
  for (const auto& q : s->mon)
    ETG_REQUIRE(q.n0 <= s->h_step && s->h_step + n_steps <= q.n0 + q.rows, ETG_ERR_STATE,
                "etg_yee3d_kernel_timing: a phasor table does not cover the steps");
  return s->dtype == ETG_F32 ? time_kernels<float>(s, n_steps, ms_h, ms_e) : time_kernels<double>(s, n_steps, ms_h, ms_e);
}

int etg_yee3d_set_option(etg_yee3d* s, int option, int64_t value) {
  ETG_REQUIRE(s && option == ETG3_OPT_FUSED && (value == 0 || value == 1), ETG_ERR_ARGUMENT,
              "etg_yee3d_set_option: bad option %d or value %lld", option, (long long)value);
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  s->fused = value == 1;
  drop_graphs(s);
  return ETG_OK;
}

}  // extern "C"
