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
// CUDA graphs of up to 32 steps; a device step counter gives every kernel its step n.
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
// so the term is d + 0 exactly and nothing is loaded. Inside, psi and the profile are read
// here, after the field loads: strip cells pay the extra round trip, the others keep few
// registers (many cells in flight per SM).
template <typename T, int W>
__device__ __forceinline__ T term(const Y3Args<T>& a, int p, int axis, int pos, int64_t idx, T d) {
  T* const psi = a.psi[p];
  const int lo = W ? a.lo_h[axis] : a.lo_e[axis], hi = W ? a.hi_h[axis] : a.hi_e[axis];
  if (psi == nullptr || (pos >= lo && pos < hi)) return add(d, T(0));
  const T* const* pr = a.prof[axis] + 3 * W;
  const T v = add(mul(pr[0][pos], psi[idx]), mul(pr[1][pos], d));
  psi[idx] = v;
  return add(mul(d, pr[2][pos]), v);
}

// H^(n-1/2) -> H^(n+1/2) from E^n: forward differences (the +1 neighbour wraps to 0 on a
// periodic axis). Hx lives at (integer x, half y, half z), Hy at (half, integer, half), Hz at
// (half, half, integer). One thread per (i, j, k), z across the lanes of a warp; all field
// loads first, then the three updates.
template <typename T>
__global__ void __launch_bounds__(256) k3_update_h(const Y3Args<T> a) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= a.m2 || j >= a.m1) return;
  const int64_t idx = i * a.si + j * a.sj + k;
  const int dk = (a.p2 && k + 1 == a.n2) ? -k : 1;
  const int dj = (a.p1 && j + 1 == a.n1) ? -j * (int)a.sj : (int)a.sj;
  const int64_t di = (a.p0 && i + 1 == a.n0) ? -(int64_t)i * a.si : a.si;
  const bool vx = j < a.n1 && k < a.n2, vy = i < a.n0 && k < a.n2, vz = i < a.n0 && j < a.n1;
  const T* __restrict__ ex = a.ex + idx;
  const T* __restrict__ ey = a.ey + idx;
  const T* __restrict__ ez = a.ez + idx;
  const T ex0 = ex[0], ey0 = ey[0], ez0 = ez[0];  // every (i, j, k) of the block is in the arrays
  const T hx0 = a.hx[idx], hy0 = a.hy[idx], hz0 = a.hz[idx];
  const T ey_k = vx ? ey[dk] : T(0), ez_j = vx ? ez[dj] : T(0);
  const T ez_i = vy ? ez[di] : T(0), ex_k = vy ? ex[dk] : T(0);
  const T ex_j = vz ? ex[dj] : T(0), ey_i = vz ? ey[di] : T(0);
  if (vx) {
    const T tz = term<T, 1>(a, 1, 2, k, idx, mul(sub(ey_k, ey0), a.inv_dz));
    const T ty = term<T, 1>(a, 0, 1, j, idx, mul(sub(ez_j, ez0), a.inv_dy));
    a.hx[idx] = add(hx0, mul(a.db, sub(tz, ty)));
  }
  if (vy) {
    const T tx = term<T, 1>(a, 3, 0, i, idx, mul(sub(ez_i, ez0), a.inv_dx));
    const T tz = term<T, 1>(a, 2, 2, k, idx, mul(sub(ex_k, ex0), a.inv_dz));
    a.hy[idx] = add(hy0, mul(a.db, sub(tx, tz)));
  }
  if (vz) {
    const T ty = term<T, 1>(a, 5, 1, j, idx, mul(sub(ex_j, ex0), a.inv_dy));
    const T tx = term<T, 1>(a, 4, 0, i, idx, mul(sub(ey_i, ey0), a.inv_dx));
    a.hz[idx] = add(hz0, mul(a.db, sub(ty, tx)));
  }
}

// E^n -> E^(n+1) from H^(n+1/2): backward differences at the integer positions off the PEC
// walls (1 .. n-1), or at all n on a periodic axis (the -1 neighbour of 0 is n-1). Tangential
// E on a wall is never written and stays as it is. All loads first, then the three updates.
template <typename T>
__global__ void __launch_bounds__(256) k3_update_e(const Y3Args<T> a) {
  const int k = blockIdx.x * 32 + threadIdx.x;
  const int j = blockIdx.y * 8 + threadIdx.y;
  const int i = blockIdx.z;
  if (k >= a.m2 || j >= a.m1) return;
  const int64_t idx = i * a.si + j * a.sj + k;
  const bool in_i = a.p0 ? i < a.n0 : (i >= 1 && i < a.n0);
  const bool in_j = a.p1 ? j < a.n1 : (j >= 1 && j < a.n1);
  const bool in_k = a.p2 ? k < a.n2 : (k >= 1 && k < a.n2);
  const int bk = (k == 0) ? a.n2 - 1 : -1;
  const int bj = (j == 0) ? (a.n1 - 1) * (int)a.sj : -(int)a.sj;
  const int64_t bi = (i == 0) ? (int64_t)(a.n0 - 1) * a.si : -a.si;
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
  if (vx) {
    const T ty = term<T, 0>(a, 6, 1, j, idx, mul(sub(hz0, hz_j), a.inv_dy));
    const T tz = term<T, 0>(a, 7, 2, k, idx, mul(sub(hy0, hy_k), a.inv_dz));
    a.ex[idx] = add(ex0, mul(cx, sub(ty, tz)));
  }
  if (vy) {
    const T tx = term<T, 0>(a, 9, 0, i, idx, mul(sub(hz0, hz_i), a.inv_dx));
    const T tz = term<T, 0>(a, 8, 2, k, idx, mul(sub(hx0, hx_k), a.inv_dz));
    a.ey[idx] = sub(ey0, mul(cy, sub(tx, tz)));
  }
  if (vz) {
    const T tx = term<T, 0>(a, 10, 0, i, idx, mul(sub(hy0, hy_i), a.inv_dx));
    const T ty = term<T, 0>(a, 11, 1, j, idx, mul(sub(hx0, hx_j), a.inv_dy));
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

__global__ void k3_step_add(int64_t* step, int g) { *step += g; }

}  // namespace
}  // namespace etg

using namespace etg;

struct etg_yee3d {
  int dtype = ETG_F32;
  int n[3] = {}, m[3] = {}, per[3] = {};
  int64_t pz = 0, sj = 0, si = 0;
  size_t elems = 0;
  void* f[Y3_NFIELD] = {};
  void* psi[Y3_NPSI] = {};
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
  std::map<int, cudaGraphExec_t> graphs;
};

namespace {

size_t esize(const etg_yee3d* s) { return s->dtype == ETG_F32 ? 4 : 8; }

// extent of field c (0..5) along each axis
void extent(const etg_yee3d* s, int c, int64_t out[3]) {
  for (int a = 0; a < 3; ++a) out[a] = kHalf[c][a] ? s->n[a] : s->m[a];
}

void drop_graphs(etg_yee3d* s) {
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
}

template <typename T>
Y3Args<T> args_of(const etg_yee3d* s) {
  Y3Args<T> a{};
  a.n0 = s->n[0], a.n1 = s->n[1], a.n2 = s->n[2];
  a.m0 = s->m[0], a.m1 = s->m[1], a.m2 = s->m[2];
  a.p0 = s->per[0], a.p1 = s->per[1], a.p2 = s->per[2];
  a.si = s->si, a.sj = s->sj;
  T* const* f = reinterpret_cast<T* const*>(s->f);
  a.ex = f[0], a.ey = f[1], a.ez = f[2], a.hx = f[3], a.hy = f[4], a.hz = f[5];
  for (int p = 0; p < Y3_NPSI; ++p) a.psi[p] = static_cast<T*>(s->psi[p]);
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
void phases_of(const etg_yee3d* s, bool magnetic, Y3SrcPhase<T>* sp, Y3MonPhase<T>* mp) {
  std::memset(sp, 0, sizeof(*sp));
  std::memset(mp, 0, sizeof(*mp));
  for (const auto& q : s->src) {
    if ((q.comp >= 3) != magnetic) continue;
    Y3Src<T>& d = sp->s[sp->n++];
    d.field = static_cast<T*>(s->f[q.comp]);
    d.idx = q.idx;
    d.table = static_cast<const T*>(q.table);
    d.n0 = q.n0, d.rows = q.rows, d.nn = q.nn;
  }
  for (const auto& q : s->mon) {
    if ((q.comp >= 3) != magnetic) continue;
    Y3Mon<T>& d = mp->m[mp->n++];
    d.acc = static_cast<T*>(q.acc);
    d.field = static_cast<const T*>(s->f[q.comp]);
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

// one step (s_off: its offset from the device counter); returns the number of launches
template <typename T>
int launch_step(const etg_yee3d* s, const Y3Args<T>& a, const Y3SrcPhase<T>& sh, const Y3MonPhase<T>& mh,
                const Y3SrcPhase<T>& se, const Y3MonPhase<T>& me, int s_off, cudaStream_t st,
                cudaEvent_t* ev = nullptr) {
  const dim3 block(32, 8), grid((s->m[2] + 31) / 32, (s->m[1] + 7) / 8, s->m[0]);
  int launches = 2;
  if (ev) cudaEventRecord(ev[0], st);
  k3_update_h<T><<<grid, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[1], st);
  if (sh.n) k3_inject<T><<<1, 32, 0, st>>>(sh, s->d_step, s_off, s->d_flag), ++launches;
  if (mh.n) k3_dft<T><<<dim3(mon_blocks(s, true), mh.n), 256, 0, st>>>(mh, s->d_step, s_off, s->d_flag), ++launches;
  if (ev) cudaEventRecord(ev[2], st);
  k3_update_e<T><<<grid, block, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[3], st);
  if (se.n) k3_inject<T><<<1, 32, 0, st>>>(se, s->d_step, s_off, s->d_flag), ++launches;
  if (me.n) k3_dft<T><<<dim3(mon_blocks(s, false), me.n), 256, 0, st>>>(me, s->d_step, s_off, s->d_flag), ++launches;
  return launches;
}

template <typename T>
int advance(etg_yee3d* s, int64_t steps) {
  const Y3Args<T> a = args_of<T>(s);
  Y3SrcPhase<T> sh, se;
  Y3MonPhase<T> mh, me;
  phases_of<T>(s, true, &sh, &mh);
  phases_of<T>(s, false, &se, &me);
  int64_t launches = 0;
  ETG_TRY_CUDA(cudaEventRecord(s->ev0, s->stream));
  const int g = Y3_GRAPH_STEPS;
  int64_t left = steps;
  if (left >= g) {
    auto it = s->graphs.find(g);
    if (it == s->graphs.end()) {
      cudaGraph_t graph = nullptr;
      ETG_TRY_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      int per = 0;
      for (int k = 0; k < g; ++k) per += launch_step<T>(s, a, sh, mh, se, me, k, s->stream);
      k3_step_add<<<1, 1, 0, s->stream>>>(s->d_step, g);
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
      it = s->graphs.emplace(g, exec).first;
      (void)per;
    }
    for (; left >= g; left -= g) {
      ETG_TRY_CUDA(cudaGraphLaunch(it->second, s->stream));
      launches += (int64_t)g * (2 + (sh.n > 0) + (mh.n > 0) + (se.n > 0) + (me.n > 0)) + 1;
    }
  }
  for (int k = 0; k < left; ++k) launches += launch_step<T>(s, a, sh, mh, se, me, k, s->stream);
  if (left) {
    k3_step_add<<<1, 1, 0, s->stream>>>(s->d_step, (int)left);
    ++launches;
  }
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
    if (kPsiAxis[p] != axis || s->psi[p]) continue;
    ETG_REQUIRE(cudaMalloc(&s->psi[p], s->elems * esize(s)) == cudaSuccess, ETG_ERR_ALLOC,
                "etg_yee3d: psi allocation of %zu bytes failed", s->elems * esize(s));
    ETG_TRY_CUDA(cudaMemsetAsync(s->psi[p], 0, s->elems * esize(s), s->stream));
  }
  return ETG_OK;
}

}  // namespace

extern "C" {

int etg_yee3d_create(etg_yee3d** out, int dtype, int nx, int ny, int nz, int periodic_mask) {
  ETG_REQUIRE(out && dtype_ok(dtype) && nx > 0 && ny > 0 && nz > 0 && periodic_mask >= 0 && periodic_mask < 8,
              ETG_ERR_ARGUMENT, "etg_yee3d_create: bad arguments (dtype %d, %d x %d x %d, periodic %d)", dtype, nx,
              ny, nz, periodic_mask);
  ETG_REQUIRE(nx < 65535 && (int64_t)(nx + 1) * (ny + 1) * (nz + 8) < (int64_t(1) << 40), ETG_ERR_ARGUMENT,
              "etg_yee3d_create: grid %d x %d x %d too large", nx, ny, nz);
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
    void** p = c < Y3_NFIELD ? &s->f[c] : &s->cb[c - Y3_NFIELD];
    if (cudaMalloc(p, s->elems * z) != cudaSuccess || cudaMemsetAsync(*p, 0, s->elems * z, s->stream) != cudaSuccess) {
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
      if (cudaMalloc(&s->prof[a][q], len[q] * z) != cudaSuccess ||
          cudaMemcpy(s->prof[a][q], dtype == ETG_F32 ? (const void*)onef.data() : (const void*)one.data(), len[q] * z,
                     cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("etg_yee3d_create: profile allocation failed");
        return fail(ETG_ERR_ALLOC);
      }
    }
    s->lo_e[a] = 0, s->hi_e[a] = s->m[a], s->lo_h[a] = 0, s->hi_h[a] = s->n[a];
  }
  if (cudaMalloc(&s->d_step, sizeof(int64_t)) != cudaSuccess || cudaMalloc(&s->d_flag, sizeof(int)) != cudaSuccess ||
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
  for (void* p : s->f) cudaFree(p);
  for (void* p : s->psi) cudaFree(p);
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
  void* dst = id < Y3_NFIELD ? s->f[id] : id < Y3_NFIELD + Y3_NPSI ? s->psi[id - Y3_NFIELD] : s->cb[c];
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
  return copy_in(s, dst, host, c);
}

int etg_yee3d_get_field(etg_yee3d* s, int id, void* host) {
  ETG_REQUIRE(s && host && id >= 0 && id < Y3_NFIELD + Y3_NPSI + Y3_NCB, ETG_ERR_ARGUMENT,
              "etg_yee3d_get_field: bad field id %d", id);
  const int c = field_comp(id);
  const void* src = id < Y3_NFIELD ? s->f[id] : id < Y3_NFIELD + Y3_NPSI ? s->psi[id - Y3_NFIELD] : s->cb[c];
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
  etg_yee3d::Src q{component, n_nodes, nullptr, nullptr, n0, rows};
  const size_t tb = (size_t)rows * n_nodes * esize(s);
  if (cudaMalloc(&q.idx, n_nodes * sizeof(int64_t)) != cudaSuccess || cudaMalloc(&q.table, tb) != cudaSuccess) {
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
  if (cudaMalloc(&q.idx, n_nodes * sizeof(int64_t)) != cudaSuccess || cudaMalloc(&q.acc, ab) != cudaSuccess ||
      cudaMalloc(&q.table, tb) != cudaSuccess) {
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
  cudaEvent_t ev[4];
  for (auto& e : ev) ETG_TRY_CUDA(cudaEventCreate(&e));
  double th = 0, te = 0;
  int rc = ETG_OK;
  for (int k = 0; k < n_steps && rc == ETG_OK; ++k) {
    if (s->dtype == ETG_F32) {
      const Y3Args<float> a = args_of<float>(s);
      Y3SrcPhase<float> sh, se;
      Y3MonPhase<float> mh, me;
      phases_of<float>(s, true, &sh, &mh);
      phases_of<float>(s, false, &se, &me);
      launch_step<float>(s, a, sh, mh, se, me, 0, s->stream, ev);
    } else {
      const Y3Args<double> a = args_of<double>(s);
      Y3SrcPhase<double> sh, se;
      Y3MonPhase<double> mh, me;
      phases_of<double>(s, true, &sh, &mh);
      phases_of<double>(s, false, &se, &me);
      launch_step<double>(s, a, sh, mh, se, me, 0, s->stream, ev);
    }
    k3_step_add<<<1, 1, 0, s->stream>>>(s->d_step, 1);
    if (cudaEventSynchronize(ev[3]) != cudaSuccess) {
      set_error("etg_yee3d_kernel_timing: %s", cudaGetErrorString(cudaGetLastError()));
      rc = ETG_ERR_CUDA;
      break;
    }
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[2], ev[3]);
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

}  // extern "C"
