// The resident simulation handle (etg_sim): HBM layout, tables, step loop, CUDA graphs.
//
// One handle is one Etalon FDTDSolver run (etalon/fdtd/solver.py:49-160) kept on the
// device: the per-step host work of the reference — computing the source delta and
// copying it to the device, building phasor rows — is replaced by tables uploaded
// once, and a block of steps is one graph launch.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "etg_sim.h"
#include "etg_tb.h"

using namespace etg;

namespace {

// Longest run of indices not marked live: [lo, hi). Everything outside is a CPML strip.
void strip_bounds(const std::vector<char>& live, int* lo, int* hi) {
  const int n = (int)live.size();
  int best_lo = 0, best_len = -1, run_lo = 0;
  for (int k = 0; k <= n; ++k) {
    if (k == n || live[k]) {
      if (k - run_lo > best_len) {
        best_len = k - run_lo;
        best_lo = run_lo;
      }
      run_lo = k + 1;
    }
  }
  *lo = best_lo;
  *hi = best_lo + std::max(best_len, 0);
}

template <typename T>
bool coefficient_live(T b, T c) {
  // psi' = b psi + c dF stays exactly +0 from +0 when c == 0 and b is positive and finite.
  return !(c == T(0)) || !(b > T(0)) || !std::isfinite((double)b);
}

void invalidate_graphs(etg_sim* s) {
  for (auto& kv : s->graphs) cudaGraphExecDestroy(kv.second);
  s->graphs.clear();
}

void update_strips(etg_sim* s) {
  std::vector<char> lx(s->nx + 1, 0), ly(s->ny + 1, 0);
  for (int k = 0; k <= s->nx; ++k) lx[k] = s->live_x[k] || s->psi_live_x[k];
  for (int k = 0; k <= s->ny; ++k) ly[k] = s->live_y[k] || s->psi_live_y[k];
  const int old[8] = {s->xs_lo, s->xs_hi, s->ys_lo, s->ys_hi, s->ux_lo, s->ux_hi, s->uy_lo, s->uy_hi};
  strip_bounds(lx, &s->xs_lo, &s->xs_hi);
  strip_bounds(ly, &s->ys_lo, &s->ys_hi);
  for (int k = 0; k <= s->nx; ++k) lx[k] = lx[k] || s->nonunit_x[k];
  for (int k = 0; k <= s->ny; ++k) ly[k] = ly[k] || s->nonunit_y[k];
  strip_bounds(lx, &s->ux_lo, &s->ux_hi);
  strip_bounds(ly, &s->uy_lo, &s->uy_hi);
  const int now[8] = {s->xs_lo, s->xs_hi, s->ys_lo, s->ys_hi, s->ux_lo, s->ux_hi, s->uy_lo, s->uy_hi};
  if (memcmp(old, now, sizeof old) != 0) {
    invalidate_graphs(s);  // the strip bounds are captured kernel parameters
    if (s->tb) tb_invalidate(s->tb);
  }
}

template <typename T>
SimArgs<T> sim_args(etg_sim* s) {
  SimArgs<T> a;
  a.nx = s->nx;
  a.ny = s->ny;
  a.P = s->P;
  a.ex = (T*)s->field[ETG_EX];
  a.ey = (T*)s->field[ETG_EY];
  a.hz = (T*)s->field[ETG_HZ];
  a.psi_ex_y = (T*)s->field[ETG_PSI_EX_Y];
  a.psi_ey_x = (T*)s->field[ETG_PSI_EY_X];
  a.psi_hz_x = (T*)s->field[ETG_PSI_HZ_X];
  a.psi_hz_y = (T*)s->field[ETG_PSI_HZ_Y];
  a.cb_ex = (const T*)s->cb[0];
  a.cb_ey = (const T*)s->cb[1];
  a.db_node = (const T*)s->db_node;
  const T** c[12] = {&a.bx_e, &a.cx_e, &a.ikx_e, &a.bx_h, &a.cx_h, &a.ikx_h,
                     &a.by_e, &a.cy_e, &a.iky_e, &a.by_h, &a.cy_h, &a.iky_h};
  for (int k = 0; k < 12; ++k) *c[k] = (const T*)s->c1d[k];
  a.db = (T)s->db;
  a.inv_dx = (T)s->inv_dx;
  a.inv_dy = (T)s->inv_dy;
  a.xs_lo = s->xs_lo;
  a.xs_hi = s->xs_hi;
  a.ys_lo = s->ys_lo;
  a.ys_hi = s->ys_hi;
  a.ux_lo = s->ux_lo;
  a.ux_hi = s->ux_hi;
  a.uy_lo = s->uy_lo;
  a.uy_hi = s->uy_hi;
  a.step = s->d_step;
  a.flag = s->d_flag;
  return a;
}

// sample_slots > 0: monitors record their samples for blocks of up to sample_slots steps
// (temporally blocked kernels) instead of accumulating in place.
template <typename T>
int build_plans(etg_sim* s, PhasePlan<T>* ph, PhasePlan<T>* pe, int64_t sample_slots = 0) {
  memset(ph, 0, sizeof *ph);
  memset(pe, 0, sizeof *pe);
  for (const Source& src : s->sources) {
    PhasePlan<T>* p = src.comp == ETG_HZ ? ph : pe;
    for (size_t k = 0; k < src.i.size(); ++k) {
      ETG_REQUIRE(p->n_src < MAX_SRC_NODES, ETG_ERR_ARGUMENT,
                  "more than %d source nodes in one half step", MAX_SRC_NODES);
      SrcDesc<T>& d = p->src[p->n_src++];
      d.table = (const T*)src.table + k;
      d.n0 = src.n0;
      d.rows = src.rows;
      d.i = (int)src.i[k];
      d.j = (int)src.j[k];
      d.stride = (int)src.i.size();
      d.comp = src.comp;
    }
  }
  if (s->trace_buf) {
    ph->trace.buf = (T*)s->trace_buf;
    ph->trace.n0 = s->trace_n0;
    ph->trace.rows = s->trace_rows;
    ph->trace.ti0 = s->trace_ti0;
    ph->trace.tnx = s->trace_tnx;
    ph->trace.tj0 = s->trace_tj0;
    ph->trace.tny = s->trace_tny;
    ph->trace.cone = s->trace_cone ? 1 : 0;
  }
  for (Monitor& m : s->monitors) {
    if (!s->monitors_on) break;
    if (sample_slots > m.samp_slots) {
      cudaFree(m.samp);
      m.samp = nullptr;
      m.samp_slots = 0;
      int rc = etg_malloc(&m.samp, (size_t)sample_slots * m.nxm * m.nym * s->esize());
      if (rc) return rc;
      m.samp_slots = sample_slots;
    }
    PhasePlan<T>* p = m.comp == ETG_HZ ? ph : pe;
    ETG_REQUIRE(p->n_mon < MAX_MONITORS, ETG_ERR_ARGUMENT,
                "more than %d monitor components in one half step", MAX_MONITORS);
    MonDesc<T>& d = p->mon[p->n_mon++];
    d.acc = (T*)m.acc;
    d.table = (const T*)m.table;
    d.samp = sample_slots > 0 ? (T*)m.samp : nullptr;
    d.n0 = m.n0;
    d.rows = m.rows;
    d.ix0 = m.ix0;
    d.nxm = m.nxm;
    d.jy0 = m.jy0;
    d.nym = m.nym;
    d.n_f = m.n_f;
    d.comp = m.comp;
  }
  return ETG_OK;
}

int check_tables(etg_sim* s, int64_t n_steps) {
  const int64_t a = s->h_step, b = s->h_step + n_steps;
  for (size_t k = 0; k < s->sources.size(); ++k) {
    const Source& src = s->sources[k];
    ETG_REQUIRE(src.n0 <= a && b <= src.n0 + src.rows, ETG_ERR_STATE,
                "source %zu has deltas for steps [%lld, %lld) but the run needs [%lld, %lld)", k,
                (long long)src.n0, (long long)(src.n0 + src.rows), (long long)a, (long long)b);
  }
  for (size_t k = 0; k < s->monitors.size(); ++k) {
    const Monitor& m = s->monitors[k];
    ETG_REQUIRE(m.n0 <= a && b <= m.n0 + m.rows, ETG_ERR_STATE,
                "monitor %zu has phasors for steps [%lld, %lld) but the run needs [%lld, %lld)", k,
                (long long)m.n0, (long long)(m.n0 + m.rows), (long long)a, (long long)b);
  }
  return ETG_OK;
}

template <typename T>
int advance_plain(etg_sim* s, int64_t n_steps) {
  PhasePlan<T> ph, pe;
  int rc = build_plans<T>(s, &ph, &pe);
  if (rc) return rc;
  SimArgs<T> a = sim_args<T>(s);
  const int64_t g = s->opt[ETG_OPT_GRAPH_STEPS];
  int64_t done = 0;
  if (g > 0 && n_steps >= g) {
    auto it = s->graphs.find(g);
    if (it == s->graphs.end()) {
      cudaGraph_t graph;
      ETG_TRY_CUDA(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
      for (int k = 0; k < g; ++k) launch_step_plain<T>(a, ph, pe, k, s->stream);
      launch_step_add<T>(a, g, s->stream);
      cudaError_t e = cudaStreamEndCapture(s->stream, &graph);
      ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
      cudaGraphExec_t exec;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
      it = s->graphs.emplace(g, exec).first;
    }
    for (; done + g <= n_steps; done += g) {
      ETG_TRY_CUDA(cudaGraphLaunch(it->second, s->stream));
      g_launches += 2 * g + 1;
    }
  }
  const int64_t rem = n_steps - done;
  for (int k = 0; k < rem; ++k) launch_step_plain<T>(a, ph, pe, k, s->stream);
  if (rem) launch_step_add<T>(a, rem, s->stream);
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

template <typename T>
int advance_dispatch(etg_sim* s, int64_t n_steps) {
  int64_t opt[10];
  memcpy(opt, s->opt, sizeof opt);
  // per-node db (TM mode): the TMA-fed kernels stage cb themselves and do not take it, so such a
  // simulation runs the plain temporally blocked kernel instead
  if (s->db_node && (opt[ETG_OPT_KERNEL] == 3 || opt[ETG_OPT_KERNEL] == 4)) opt[ETG_OPT_KERNEL] = 2;
  const int64_t kernel = opt[ETG_OPT_KERNEL];
  if (kernel == 2 || kernel == 3 || kernel == 4 || (kernel == 0 && tb_supported<T>(s->nx, s->ny))) {
    PhasePlan<T> ph, pe;  // the TMA kernel accumulates in place; the others sample per block
    int rc = build_plans<T>(s, &ph, &pe, kernel == 3 ? 0 : sim_sample_slots(s));
    if (rc) return rc;
    if (!s->tb) s->tb = tb_create();
    return tb_advance<T>(s->tb, sim_args<T>(s), ph, pe, n_steps, opt, s->stream);
  }
  return advance_plain<T>(s, n_steps);
}

int copy_field_in(etg_sim* s, void* dst, const void* host, int64_t rows, int64_t cols) {
  ETG_TRY_CUDA(cudaMemcpy2DAsync(dst, s->P * s->esize(), host, cols * s->esize(), cols * s->esize(),
                                 rows, cudaMemcpyHostToDevice, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

template <typename T>
void mark_nonzero(const T* a, int64_t rows, int64_t cols, std::vector<char>& by_row,
                  std::vector<char>& by_col) {
  for (int64_t r = 0; r < rows; ++r)
    for (int64_t c = 0; c < cols; ++c) {
      const T v = a[r * cols + c];
      if (!(v == T(0)) || std::signbit((double)v)) {
        by_row[r] = 1;
        by_col[c] = 1;
      }
    }
}

int zero_device(etg_sim* s) {
  for (int f = 0; f < 7; ++f)
    ETG_TRY_CUDA(cudaMemsetAsync(s->field[f], 0, s->rows * s->P * s->esize(), s->stream));
  for (Monitor& m : s->monitors)
    ETG_TRY_CUDA(cudaMemsetAsync(m.acc, 0, (size_t)2 * m.n_f * m.nxm * m.nym * s->esize(), s->stream));
  ETG_TRY_CUDA(cudaMemsetAsync(s->d_step, 0, sizeof(int64_t), s->stream));
  ETG_TRY_CUDA(cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  s->h_step = 0;
  return ETG_OK;
}

}  // namespace

namespace etg {

int sim_advance_internal(etg_sim* s, int64_t n_steps) {
  if (n_steps == 0) return ETG_OK;
  int rc = check_tables(s, n_steps);
  if (rc) return rc;
  s->psi_dirty = true;
  rc = s->dtype == ETG_F32 ? advance_dispatch<float>(s, n_steps) : advance_dispatch<double>(s, n_steps);
  if (rc) return rc;
  s->h_step += n_steps;
  return ETG_OK;
}

void sim_invalidate(etg_sim* s) {
  invalidate_graphs(s);
  if (s->tb) tb_invalidate(s->tb);
}

template <typename T>
SimArgs<T> sim_args_export(etg_sim* s) {
  return sim_args<T>(s);
}

template <typename T>
int sim_plans_export(etg_sim* s, PhasePlan<T>* ph, PhasePlan<T>* pe, int64_t sample_slots) {
  return build_plans<T>(s, ph, pe, sample_slots);
}

int64_t sim_sample_slots(const etg_sim* s) { return std::max<int64_t>(16, s->opt[ETG_OPT_GRAPH_STEPS]); }

int sim_check_tables(etg_sim* s, int64_t n_steps) { return check_tables(s, n_steps); }

template SimArgs<float> sim_args_export<float>(etg_sim*);
template SimArgs<double> sim_args_export<double>(etg_sim*);
template int sim_plans_export<float>(etg_sim*, PhasePlan<float>*, PhasePlan<float>*, int64_t);
template int sim_plans_export<double>(etg_sim*, PhasePlan<double>*, PhasePlan<double>*, int64_t);

}  // namespace etg

extern "C" {

int etg_sim_create(etg_sim** out, int dtype, int nx, int ny) {
  ETG_REQUIRE(out, ETG_ERR_ARGUMENT, "etg_sim_create: null output pointer");
  ETG_REQUIRE(dtype_ok(dtype), ETG_ERR_ARGUMENT, "etg_sim_create: dtype must be 4 or 8, got %d", dtype);
  // rows: the one-step and adjoint kernels put 4 x rows per block on gridDim.y (at most 65535)
  ETG_REQUIRE(nx >= 2 && ny >= 2 && nx <= 262136 && ny < (1 << 28), ETG_ERR_ARGUMENT,
              "etg_sim_create: grid %d x %d out of range (2 <= nx <= 262136, 2 <= ny < 2^28)", nx, ny);
  if (fault_injected("etg_sim_create")) return ETG_ERR_INJECTED;
  *out = nullptr;
  etg_sim* s = new etg_sim;
  s->dtype = dtype;
  s->nx = nx;
  s->ny = ny;
  s->P = ((int64_t)ny + 1 + 31) / 32 * 32;
  s->rows = (int64_t)nx + 2;
  s->live_x.assign(nx + 1, 0);
  s->live_y.assign(ny + 1, 0);
  s->psi_live_x.assign(nx + 1, 0);
  s->psi_live_y.assign(ny + 1, 0);
  s->nonunit_x.assign(nx + 1, 1);
  s->nonunit_y.assign(ny + 1, 1);
  int rc = ETG_OK;
  auto fail = [&](int code) {
    etg_sim_destroy(s);
    return code;
  };
  const size_t plane = (size_t)s->rows * s->P * s->esize();
  for (int f = 0; f < 7 && rc == ETG_OK; ++f) rc = etg_malloc(&s->field[f], plane);
  for (int k = 0; k < 2 && rc == ETG_OK; ++k) rc = etg_malloc(&s->cb[k], plane);
  const int64_t len[12] = {nx + 1, nx + 1, nx + 1, nx, nx, nx, ny + 1, ny + 1, ny + 1, ny, ny, ny};
  for (int k = 0; k < 12 && rc == ETG_OK; ++k) rc = etg_malloc(&s->c1d[k], (len[k] + 8) * s->esize());
  if (rc == ETG_OK) rc = etg_malloc((void**)&s->d_step, sizeof(int64_t));
  if (rc == ETG_OK) rc = etg_malloc((void**)&s->d_flag, sizeof(int));
  if (rc) return fail(rc);
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&s->ev0) != cudaSuccess || cudaEventCreate(&s->ev1) != cudaSuccess) {
    set_error("etg_sim_create: stream/event creation failed: %s", cudaGetErrorString(cudaGetLastError()));
    return fail(ETG_ERR_CUDA);
  }
  for (int k = 0; k < 2; ++k)
    if (cudaMemsetAsync(s->cb[k], 0, plane, s->stream) != cudaSuccess) return fail(ETG_ERR_CUDA);
  for (int k = 0; k < 12; ++k)
    if (cudaMemsetAsync(s->c1d[k], 0, (len[k] + 8) * s->esize(), s->stream) != cudaSuccess)
      return fail(ETG_ERR_CUDA);
  rc = zero_device(s);
  if (rc) return fail(rc);
  update_strips(s);
  *out = s;
  return ETG_OK;
}

int etg_sim_destroy(etg_sim* s) {
  if (!s) return ETG_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  invalidate_graphs(s);
  if (s->tb) tb_destroy(s->tb);
  for (void* p : s->field) cudaFree(p);
  for (void* p : s->cb) cudaFree(p);
  cudaFree(s->db_node);
  for (void* p : s->c1d) cudaFree(p);
  for (Source& src : s->sources) cudaFree(src.table);
  for (Monitor& m : s->monitors) {
    cudaFree(m.acc);
    cudaFree(m.table);
    cudaFree(m.samp);
  }
  cudaFree(s->d_step);
  cudaFree(s->d_flag);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return ETG_OK;
}

int etg_sim_set_coefficients(etg_sim* s, const void* cb_ex, const void* cb_ey, const void* bx_e,
                             const void* cx_e, const void* ikx_e, const void* bx_h,
                             const void* cx_h, const void* ikx_h, const void* by_e,
                             const void* cy_e, const void* iky_e, const void* by_h,
                             const void* cy_h, const void* iky_h, double db, double inv_dx,
                             double inv_dy) {
  ETG_REQUIRE(s && cb_ex && cb_ey, ETG_ERR_ARGUMENT, "etg_sim_set_coefficients: null argument");
  int rc = copy_field_in(s, s->cb[0], cb_ex, s->nx, s->ny + 1);
  if (rc == ETG_OK) rc = copy_field_in(s, s->cb[1], cb_ey, s->nx + 1, s->ny);
  if (rc) return rc;
  const void* c[12] = {bx_e, cx_e, ikx_e, bx_h, cx_h, ikx_h, by_e, cy_e, iky_e, by_h, cy_h, iky_h};
  const int64_t len[12] = {s->nx + 1, s->nx + 1, s->nx + 1, s->nx, s->nx, s->nx,
                           s->ny + 1, s->ny + 1, s->ny + 1, s->ny, s->ny, s->ny};
  for (int k = 0; k < 12; ++k) {
    ETG_REQUIRE(c[k], ETG_ERR_ARGUMENT, "etg_sim_set_coefficients: null 1D array %d", k);
    ETG_TRY_CUDA(cudaMemcpy(s->c1d[k], c[k], len[k] * s->esize(), cudaMemcpyHostToDevice));
  }
  // psi may be non-zero wherever it was live since the last reset: those rows and columns
  // stay strips whatever the new coefficients say
  if (s->psi_dirty) {
    for (int k = 0; k <= s->nx; ++k) s->psi_live_x[k] |= s->live_x[k];
    for (int k = 0; k <= s->ny; ++k) s->psi_live_y[k] |= s->live_y[k];
  }
  // live CPML rows/columns: psi_hz_x (h, i < nx), psi_ey_x (e, 1 <= i <= nx-1), same for y
  std::fill(s->live_x.begin(), s->live_x.end(), 0);
  std::fill(s->live_y.begin(), s->live_y.end(), 0);
  std::fill(s->nonunit_x.begin(), s->nonunit_x.end(), 0);
  std::fill(s->nonunit_y.begin(), s->nonunit_y.end(), 0);
  auto scan = [&](auto tag) {
    using T = decltype(tag);
    const T *bxe = (const T*)bx_e, *cxe = (const T*)cx_e, *bxh = (const T*)bx_h, *cxh = (const T*)cx_h;
    const T *bye = (const T*)by_e, *cye = (const T*)cy_e, *byh = (const T*)by_h, *cyh = (const T*)cy_h;
    const T *kxe = (const T*)ikx_e, *kxh = (const T*)ikx_h, *kye = (const T*)iky_e, *kyh = (const T*)iky_h;
    for (int i = 0; i < s->nx; ++i) {
      s->live_x[i] |= coefficient_live(bxh[i], cxh[i]);
      s->nonunit_x[i] |= !(kxh[i] == T(1));
    }
    for (int i = 1; i < s->nx; ++i) {
      s->live_x[i] |= coefficient_live(bxe[i], cxe[i]);
      s->nonunit_x[i] |= !(kxe[i] == T(1));
    }
    for (int j = 0; j < s->ny; ++j) {
      s->live_y[j] |= coefficient_live(byh[j], cyh[j]);
      s->nonunit_y[j] |= !(kyh[j] == T(1));
    }
    for (int j = 1; j < s->ny; ++j) {
      s->live_y[j] |= coefficient_live(bye[j], cye[j]);
      s->nonunit_y[j] |= !(kye[j] == T(1));
    }
  };
  if (s->dtype == ETG_F32) scan(float{}); else scan(double{});
  if (s->db != db || s->inv_dx != inv_dx || s->inv_dy != inv_dy) {
    invalidate_graphs(s);  // captured kernel parameters
    if (s->tb) tb_invalidate(s->tb);
  }
  s->db = db;
  s->inv_dx = inv_dx;
  s->inv_dy = inv_dy;
  s->have_coeffs = true;
  update_strips(s);
  return ETG_OK;
}

int etg_sim_set_cb_window(etg_sim* s, int which, int i0, int rows, int j0, int cols, const void* host) {
  ETG_REQUIRE(s && host && (which == 0 || which == 1) && rows > 0 && cols > 0, ETG_ERR_ARGUMENT,
              "etg_sim_set_cb_window: bad arguments");
  const int64_t nr = which == 1 ? s->nx + 1 : s->nx, nc = which == 0 ? s->ny + 1 : s->ny;
  ETG_REQUIRE(i0 >= 0 && j0 >= 0 && i0 + rows <= nr && j0 + cols <= nc, ETG_ERR_ARGUMENT,
              "etg_sim_set_cb_window: window [%d,%d)x[%d,%d) outside the %lld x %lld array", i0, i0 + rows,
              j0, j0 + cols, (long long)nr, (long long)nc);
  char* dst = (char*)s->cb[which] + ((int64_t)i0 * s->P + j0) * s->esize();
  ETG_TRY_CUDA(cudaMemcpy2DAsync(dst, s->P * s->esize(), host, cols * s->esize(), cols * s->esize(), rows,
                                 cudaMemcpyHostToDevice, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int etg_sim_set_db_nodes(etg_sim* s, const void* host) {
  ETG_REQUIRE(s && host, ETG_ERR_ARGUMENT, "etg_sim_set_db_nodes: bad arguments");
  if (!s->db_node) {
    const size_t bytes = (size_t)s->rows * s->P * s->esize();
    ETG_TRY_CUDA(cudaMalloc(&s->db_node, bytes));
    ETG_TRY_CUDA(cudaMemset(s->db_node, 0, bytes));
    invalidate_graphs(s);  // the pointer is a captured kernel parameter
    if (s->tb) tb_invalidate(s->tb);
  }
  return copy_field_in(s, s->db_node, host, s->nx, s->ny);
}

int etg_sim_add_source(etg_sim* s, int component, int n_nodes, const int64_t* i, const int64_t* j,
                       int64_t n0, int64_t rows, const void* table) {
  ETG_REQUIRE(s && i && j && table && n_nodes > 0 && rows >= 0, ETG_ERR_ARGUMENT,
              "etg_sim_add_source: bad arguments");
  ETG_REQUIRE(component == ETG_EX || component == ETG_EY || component == ETG_HZ, ETG_ERR_ARGUMENT,
              "etg_sim_add_source: component must be ETG_EX, ETG_EY or ETG_HZ");
  const int64_t nr = component == ETG_EY ? s->nx + 1 : s->nx;
  const int64_t nc = component == ETG_EX ? s->ny + 1 : s->ny;
  for (int k = 0; k < n_nodes; ++k)
    ETG_REQUIRE(i[k] >= 0 && i[k] < nr && j[k] >= 0 && j[k] < nc, ETG_ERR_ARGUMENT,
                "etg_sim_add_source: node (%lld, %lld) outside the %lld x %lld array",
                (long long)i[k], (long long)j[k], (long long)nr, (long long)nc);
  if (s->tb) tb_invalidate(s->tb);
  Source src;
  src.comp = component;
  src.i.assign(i, i + n_nodes);
  src.j.assign(j, j + n_nodes);
  src.n0 = n0;
  src.rows = rows;
  const size_t bytes = (size_t)std::max<int64_t>(rows, 1) * n_nodes * s->esize();
  int rc = etg_malloc(&src.table, bytes);
  if (rc) return rc;
  if (rows) ETG_TRY_CUDA(cudaMemcpy(src.table, table, rows * n_nodes * s->esize(), cudaMemcpyHostToDevice));
  s->sources.push_back(src);
  invalidate_graphs(s);
  return ETG_OK;
}

int etg_sim_set_deltas(etg_sim* s, int source, int64_t n0, int64_t rows, const void* table) {
  ETG_REQUIRE(s && source >= 0 && source < (int)s->sources.size() && rows >= 0 && table,
              ETG_ERR_ARGUMENT, "etg_sim_set_deltas: bad source %d", source);
  Source& src = s->sources[source];
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  const bool same = rows == src.rows && n0 == src.n0;  // captured graphs stay valid
  if (rows > src.rows) {
    cudaFree(src.table);
    src.table = nullptr;
    int rc = etg_malloc(&src.table, rows * src.i.size() * s->esize());
    if (rc) return rc;
  }
  ETG_TRY_CUDA(cudaMemcpy(src.table, table, rows * src.i.size() * s->esize(), cudaMemcpyHostToDevice));
  src.n0 = n0;
  src.rows = rows;
  if (!same) {
    invalidate_graphs(s);
    if (s->tb) tb_invalidate(s->tb);
  }
  return ETG_OK;
}

int etg_sim_add_monitor(etg_sim* s, int component, int ix0, int nxm, int jy0, int nym, int n_f,
                        int64_t n0, int64_t rows, const void* table, int* monitor) {
  ETG_REQUIRE(s && table && monitor && n_f > 0 && nxm > 0 && nym > 0 && rows >= 0,
              ETG_ERR_ARGUMENT, "etg_sim_add_monitor: bad arguments");
  ETG_REQUIRE(component == ETG_EX || component == ETG_EY || component == ETG_HZ, ETG_ERR_ARGUMENT,
              "etg_sim_add_monitor: component must be ETG_EX, ETG_EY or ETG_HZ");
  const int64_t nr = component == ETG_EY ? s->nx + 1 : s->nx;
  const int64_t nc = component == ETG_EX ? s->ny + 1 : s->ny;
  ETG_REQUIRE(ix0 >= 0 && jy0 >= 0 && ix0 + nxm <= nr && jy0 + nym <= nc, ETG_ERR_ARGUMENT,
              "etg_sim_add_monitor: rectangle [%d,%d)x[%d,%d) outside the %lld x %lld array", ix0,
              ix0 + nxm, jy0, jy0 + nym, (long long)nr, (long long)nc);
  if (s->tb) tb_invalidate(s->tb);
  Monitor m{component, ix0, nxm, jy0, nym, n_f};
  m.n0 = n0;
  m.rows = rows;
  const size_t acc_bytes = (size_t)2 * n_f * nxm * nym * s->esize();
  int rc = etg_malloc(&m.acc, acc_bytes);
  if (rc == ETG_OK) rc = etg_malloc(&m.table, (size_t)2 * std::max<int64_t>(rows, 1) * n_f * s->esize());
  if (rc) {
    cudaFree(m.acc);
    return rc;
  }
  ETG_TRY_CUDA(cudaMemset(m.acc, 0, acc_bytes));
  if (rows) ETG_TRY_CUDA(cudaMemcpy(m.table, table, 2 * rows * n_f * s->esize(), cudaMemcpyHostToDevice));
  *monitor = (int)s->monitors.size();
  s->monitors.push_back(m);
  invalidate_graphs(s);
  return ETG_OK;
}

int etg_sim_set_phasors(etg_sim* s, int monitor, int64_t n0, int64_t rows, const void* table) {
  ETG_REQUIRE(s && monitor >= 0 && monitor < (int)s->monitors.size() && rows >= 0 && table,
              ETG_ERR_ARGUMENT, "etg_sim_set_phasors: bad monitor %d", monitor);
  Monitor& m = s->monitors[monitor];
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  const bool same = rows == m.rows && n0 == m.n0;  // captured graphs stay valid
  if (rows > m.rows) {
    cudaFree(m.table);
    m.table = nullptr;
    int rc = etg_malloc(&m.table, (size_t)2 * rows * m.n_f * s->esize());
    if (rc) return rc;
  }
  ETG_TRY_CUDA(cudaMemcpy(m.table, table, 2 * rows * m.n_f * s->esize(), cudaMemcpyHostToDevice));
  m.n0 = n0;
  m.rows = rows;
  if (!same) {
    invalidate_graphs(s);
    if (s->tb) tb_invalidate(s->tb);
  }
  return ETG_OK;
}

int etg_sim_set_field(etg_sim* s, int f, const void* host) {
  ETG_REQUIRE(s && host && f >= 0 && f < 7, ETG_ERR_ARGUMENT, "etg_sim_set_field: bad field %d", f);
  const int64_t r = s->field_rows(f), c = s->field_cols(f);
  int rc = copy_field_in(s, s->field[f], host, r, c);
  if (rc) return rc;
  if (f >= ETG_PSI_EX_Y) {  // uploaded psi widens the strips to wherever it is non-zero
    std::vector<char> rows_nz(r, 0), cols_nz(c, 0);
    if (s->dtype == ETG_F32) mark_nonzero((const float*)host, r, c, rows_nz, cols_nz);
    else mark_nonzero((const double*)host, r, c, rows_nz, cols_nz);
    if (f == ETG_PSI_HZ_X || f == ETG_PSI_EY_X)
      for (int64_t k = 0; k < r; ++k) s->psi_live_x[k] |= rows_nz[k];
    else
      for (int64_t k = 0; k < c; ++k) s->psi_live_y[k] |= cols_nz[k];
    update_strips(s);
  }
  return ETG_OK;
}

int etg_sim_get_field(etg_sim* s, int f, void* host) {
  ETG_REQUIRE(s && host && f >= 0 && f < 7, ETG_ERR_ARGUMENT, "etg_sim_get_field: bad field %d", f);
  const int64_t r = s->field_rows(f), c = s->field_cols(f);
  ETG_TRY_CUDA(cudaMemcpy2DAsync(host, c * s->esize(), s->field[f], s->P * s->esize(), c * s->esize(),
                                 r, cudaMemcpyDeviceToHost, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int etg_sim_device_array(etg_sim* s, int array, void** ptr, int64_t* pitch) {
  ETG_REQUIRE(s && ptr && pitch && array >= 0 && array < 9, ETG_ERR_ARGUMENT,
              "etg_sim_device_array: bad array %d", array);
  *ptr = array < 7 ? (void*)s->field[array] : (void*)s->cb[array - 7];
  *pitch = s->P;
  return ETG_OK;
}

int etg_sim_get_dft(etg_sim* s, int monitor, void* host) {
  ETG_REQUIRE(s && host && monitor >= 0 && monitor < (int)s->monitors.size(), ETG_ERR_ARGUMENT,
              "etg_sim_get_dft: bad monitor %d", monitor);
  const Monitor& m = s->monitors[monitor];
  ETG_TRY_CUDA(cudaMemcpyAsync(host, m.acc, (size_t)2 * m.n_f * m.nxm * m.nym * s->esize(),
                               cudaMemcpyDeviceToHost, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int etg_sim_set_dft(etg_sim* s, int monitor, const void* host) {
  ETG_REQUIRE(s && host && monitor >= 0 && monitor < (int)s->monitors.size(), ETG_ERR_ARGUMENT,
              "etg_sim_set_dft: bad monitor %d", monitor);
  const Monitor& m = s->monitors[monitor];
  ETG_TRY_CUDA(cudaMemcpyAsync(m.acc, host, (size_t)2 * m.n_f * m.nxm * m.nym * s->esize(),
                               cudaMemcpyHostToDevice, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  return ETG_OK;
}

int etg_sim_reset(etg_sim* s) {
  ETG_REQUIRE(s, ETG_ERR_ARGUMENT, "etg_sim_reset: null handle");
  s->psi_dirty = false;
  std::fill(s->psi_live_x.begin(), s->psi_live_x.end(), 0);
  std::fill(s->psi_live_y.begin(), s->psi_live_y.end(), 0);
  update_strips(s);
  return zero_device(s);
}

int etg_sim_advance(etg_sim* s, int64_t n_steps) {
  ETG_REQUIRE(s && n_steps >= 0, ETG_ERR_ARGUMENT, "etg_sim_advance: bad arguments");
  ETG_REQUIRE(s->have_coeffs, ETG_ERR_STATE, "etg_sim_advance: coefficients not set");
  if (fault_injected("etg_sim_advance")) return ETG_ERR_INJECTED;
  if (n_steps == 0) return ETG_OK;
  int rc = check_tables(s, n_steps);
  if (rc) return rc;
  const bool timing = s->opt[ETG_OPT_TIMING] != 0;
  const int64_t launches0 = g_launches;
  if (timing) ETG_TRY_CUDA(cudaEventRecord(s->ev0, s->stream));
  s->psi_dirty = true;
  rc = s->dtype == ETG_F32 ? advance_dispatch<float>(s, n_steps) : advance_dispatch<double>(s, n_steps);
  if (rc) return rc;
  if (s->opt[ETG_OPT_CHECK_FINITE]) {
    if (s->dtype == ETG_F32) launch_check_finite<float>(sim_args<float>(s), s->stream);
    else launch_check_finite<double>(sim_args<double>(s), s->stream);
    ETG_LAUNCH_CHECK();
  }
  if (timing) {
    ETG_TRY_CUDA(cudaEventRecord(s->ev1, s->stream));
    ETG_TRY_CUDA(cudaEventSynchronize(s->ev1));
    float ms = 0;
    ETG_TRY_CUDA(cudaEventElapsedTime(&ms, s->ev0, s->ev1));
    s->last_ms = ms;
  }
  s->last_launches = g_launches - launches0;
  s->h_step += n_steps;
  return ETG_OK;
}

int etg_sim_step_index(etg_sim* s, int64_t* n) {
  ETG_REQUIRE(s && n, ETG_ERR_ARGUMENT, "etg_sim_step_index: null argument");
  *n = s->h_step;
  return ETG_OK;
}

int etg_sim_set_step_index(etg_sim* s, int64_t n) {
  ETG_REQUIRE(s && n >= 0, ETG_ERR_ARGUMENT, "etg_sim_set_step_index: bad arguments");
  ETG_TRY_CUDA(cudaMemcpyAsync(s->d_step, &n, sizeof n, cudaMemcpyHostToDevice, s->stream));
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  s->h_step = n;
  return ETG_OK;
}

int etg_sim_synchronize(etg_sim* s) {
  ETG_REQUIRE(s, ETG_ERR_ARGUMENT, "etg_sim_synchronize: null handle");
  ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));
  int flag = 0;
  ETG_TRY_CUDA(cudaMemcpy(&flag, s->d_flag, sizeof flag, cudaMemcpyDeviceToHost));
  if (flag) {
    ETG_TRY_CUDA(cudaMemset(s->d_flag, 0, sizeof(int)));
    if (flag & ERRBIT_TIMEOUT) {
      set_error("a bounded device-side wait gave up (flags 0x%x)", flag);
      return ETG_ERR_TIMEOUT;
    }
    if (flag & ERRBIT_TABLE) {
      set_error("a source or phasor table did not cover a step (flags 0x%x)", flag);
      return ETG_ERR_STATE;
    }
    if (flag & ERRBIT_NONFINITE) {
      set_error("a field became NaN or Inf (flags 0x%x)", flag);
      return ETG_ERR_NONFINITE;
    }
  }
  return ETG_OK;
}

int etg_sim_set_option(etg_sim* s, int option, int64_t value) {
  ETG_REQUIRE(s && option >= 0 && option < 9, ETG_ERR_ARGUMENT, "etg_sim_set_option: bad option %d", option);
  ETG_REQUIRE(value >= 0, ETG_ERR_ARGUMENT, "etg_sim_set_option: negative value");
  s->opt[option] = value;
  invalidate_graphs(s);
  if (s->tb) tb_invalidate(s->tb);
  return ETG_OK;
}

int etg_sim_get_option(etg_sim* s, int option, int64_t* value) {
  ETG_REQUIRE(s && value && option >= 0 && option < 10, ETG_ERR_ARGUMENT, "etg_sim_get_option: bad option");
  if (option == ETG_OPT_TB_SEGMENTS_USED) {  // read-only: column segments of the current tile list
    *value = s->tb ? tb_segments(s->tb) : 0;
    return ETG_OK;
  }
  *value = s->opt[option];
  if (*value == 0 && option == ETG_OPT_TB_WARPS) *value = 8;
  if (*value == 0 && (option == ETG_OPT_TB_DEPTH || option == ETG_OPT_TILE_ROWS || option == ETG_OPT_TILE_COLS)) {
    int er, ec, k;  // the default tile shape of this dtype
    tb_default_shape(s->dtype, &er, &ec, &k, (int)s->opt[ETG_OPT_KERNEL]);
    *value = option == ETG_OPT_TB_DEPTH ? k : option == ETG_OPT_TILE_ROWS ? er : ec;
  }
  return ETG_OK;
}

int etg_sim_kernel_timing(etg_sim* s, double* ms, int64_t* launches, int64_t* cells) {
  ETG_REQUIRE(s && ms && launches && cells, ETG_ERR_ARGUMENT, "etg_sim_kernel_timing: bad arguments");
  tb_kernel_timing(s->tb, ms, launches, cells);
  return ETG_OK;
}

int etg_sim_last_timing(etg_sim* s, double* ms, int64_t* launches) {
  ETG_REQUIRE(s, ETG_ERR_ARGUMENT, "etg_sim_last_timing: null handle");
  if (ms) *ms = s->last_ms;
  if (launches) *launches = s->last_launches;
  return ETG_OK;
}

}  // extern "C"
