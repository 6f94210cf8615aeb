// Batched stepping of many resident simulations (no counterpart in Etalon, which runs one
// FDTDSolver per simulation): one launch pair per K steps advances every simulation of the
// batch, whatever its size. Each tile names its simulation; per-simulation arguments, second
// buffers and source/monitor plans live in device memory (BatchSim). Blocks of steps are CUDA
// graphs, as for a single simulation, and every simulation's result is bit-identical to its
// own run (the tiles compute exactly what the single-simulation kernels compute).
#include <algorithm>
#include <cstring>
#include <vector>

#include "etg_tb.h"

using namespace etg;

struct etg_batch {
  std::vector<etg_sim*> sims;
  int dtype = ETG_F32;
  std::vector<void*> alt;          // per simulation: 7 planes of the second buffer
  std::vector<size_t> alt_bytes;
  void* d_sims = nullptr;          // BatchSim<T>[n]
  std::vector<unsigned char> h_sims;
  std::vector<int4> h_tiles;
  int4* d_tiles = nullptr;
  int n_inner = 0, n_pml = 0, tiles_er = 0, tiles_k = 0;
  int n_hot = 0;  // leading interior tiles with a source, monitor or trace node (the others: lean kernel)
  std::vector<std::vector<int4>> hot_seen;  // per simulation: every such rectangle seen so far
  int64_t dft_work = 0;  // largest sampled monitor (frequencies x nodes) of any simulation
  int dft_mon = 0;       // most monitor components of any simulation
  int64_t** d_steps = nullptr;     // each simulation's step counter
  cudaStream_t stream = nullptr, side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, ev0 = nullptr, ev1 = nullptr, done = nullptr;
  cudaStream_t sides[4] = {};  // one branch per CPML kind, one for the interior tiles with a plan
  cudaEvent_t joins[4] = {};
  int n_kind[6] = {};  // CPML tiles of each kind, then the leading ones of each with a plan
  int64_t opt[8] = {0, 0, 32, 0, 0, 0, 0, 0};
  std::map<int64_t, cudaGraphExec_t> graphs;
  double last_ms = 0;
  int64_t last_launches = 0;
};

namespace {

__global__ void k_batch_step_add(int64_t* const* steps, int n, int64_t k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) *steps[i] += k;
}

void drop_graphs(etg_batch* b) {
  for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
  b->graphs.clear();
}

// Upload the per-simulation arguments when they changed (graphs read them from device
// memory, so they stay valid) and the tile list when it changed (graphs are rebuilt then:
// *changed).
template <typename T>
int refresh(etg_batch* b, int ER, int K, bool* changed) {
  const int n = (int)b->sims.size();
  ETG_TRY_CUDA(cudaStreamSynchronize(b->stream));  // no launch still reads the arguments
  b->dft_work = 0;
  b->dft_mon = 0;
  std::vector<unsigned char> host((size_t)n * sizeof(BatchSim<T>));
  for (int k = 0; k < n; ++k) {
    etg_sim* s = b->sims[k];
    BatchSim<T> e;
    memset(&e, 0, sizeof e);
    const size_t bytes = (size_t)(s->nx + 2) * s->P * sizeof(T);
    if (b->alt_bytes[k] != bytes) {
      cudaFree(b->alt[k]);
      b->alt[k] = nullptr;
      int rc = etg_malloc(&b->alt[k], 7 * bytes);
      if (rc) return rc;
      ETG_TRY_CUDA(cudaMemset(b->alt[k], 0, 7 * bytes));
      b->alt_bytes[k] = bytes;
    }
    const SimArgs<T> a = sim_args_export<T>(s);
    SimArgs<T> bb = a;
    T** bp[7] = {&bb.ex, &bb.ey, &bb.hz, &bb.psi_ex_y, &bb.psi_ey_x, &bb.psi_hz_x, &bb.psi_hz_y};
    for (int f = 0; f < 7; ++f) *bp[f] = (T*)((char*)b->alt[k] + f * bytes);
    e.src[0] = a;
    e.src[1] = bb;
    e.dst[0] = TBDst<T>{bb.ex, bb.ey, bb.hz, bb.psi_ex_y, bb.psi_ey_x, bb.psi_hz_x, bb.psi_hz_y};
    e.dst[1] = TBDst<T>{a.ex, a.ey, a.hz, a.psi_ex_y, a.psi_ey_x, a.psi_hz_x, a.psi_hz_y};
    int rc = sim_plans_export<T>(s, &e.ph, &e.pe, std::max<int64_t>(16, b->opt[ETG_OPT_GRAPH_STEPS]));
    if (rc) return rc;
    memcpy(host.data() + (size_t)k * sizeof e, &e, sizeof e);
    b->dft_mon = std::max(b->dft_mon, e.ph.n_mon + e.pe.n_mon);
    for (int m = 0; m < e.ph.n_mon + e.pe.n_mon; ++m) {
      const MonDesc<T>& d = m < e.ph.n_mon ? e.ph.mon[m] : e.pe.mon[m - e.ph.n_mon];
      if (d.samp) b->dft_work = std::max<int64_t>(b->dft_work, (int64_t)d.nxm * d.nym * d.n_f);
    }
  }
  *changed = false;
  if (host != b->h_sims) {
    if (!b->d_sims) {
      int rc = etg_malloc(&b->d_sims, host.size());
      if (rc) return rc;
    }
    ETG_TRY_CUDA(cudaMemcpy(b->d_sims, host.data(), host.size(), cudaMemcpyHostToDevice));
    b->h_sims.swap(host);
  }
  {
    // interior tiles holding a source, monitor or trace node (every simulation's) lead the
    // interior list and run the kernel with the per-step plan code; the rest run the lean one
    std::vector<int4> inner, cold;
    std::vector<std::pair<int4, bool>> pml;  // CPML tiles and whether they hold a plan node
    for (int k = 0; k < n; ++k) {
      etg_sim* s = b->sims[k];
      PhasePlan<T> ph, pe;
      sim_plans_export<T>(s, &ph, &pe);
      std::vector<int4> hot;
      for (const PhasePlan<T>* p : {&ph, &pe}) {
        for (int q = 0; q < p->n_src; ++q) hot.push_back(make_int4(p->src[q].i, p->src[q].j, p->src[q].i + 1, p->src[q].j + 1));
        for (int q = 0; q < p->n_mon; ++q)
          hot.push_back(make_int4(p->mon[q].ix0, p->mon[q].jy0, p->mon[q].ix0 + p->mon[q].nxm, p->mon[q].jy0 + p->mon[q].nym));
      }
      if (ph.trace.buf)
        hot.push_back(make_int4(ph.trace.ti0, ph.trace.tj0, ph.trace.ti0 + ph.trace.tnx, ph.trace.tj0 + ph.trace.tny));
      // the union of those seen so far: runs with and without monitors or traces keep one list
      if ((int)b->hot_seen.size() != n) b->hot_seen.assign(n, {});
      tb_hot_union(&b->hot_seen[k], hot, 1024);
      hot = b->hot_seen[k];
      std::vector<int2> t;
      int ni = 0, nh = 0, kh[3] = {0, 0, 0};
      const int EC = 32 * (sizeof(T) == 4 ? 4 : 2);
      tb_split_tiles(s->nx, s->ny, s->ux_lo, s->ux_hi, s->uy_lo, s->uy_hi, ER, EC, K, hot, &t, &ni, &nh, kh);
      int seen_of_kind[3] = {0, 0, 0};  // this simulation's CPML tiles come grouped by kind, plan tiles first
      for (int q = 0; q < (int)t.size(); ++q) {
        const int r0 = tb_tile_row(t[q]), c0 = t[q].y;  // output rows [r0, r0+ER-2K), columns [c0, c0+EC-2K)
        const int kind = tb_tile_kind(t[q]);
        const bool planned = q >= ni && seen_of_kind[kind - 1]++ < kh[kind - 1];
        if (r0 >= s->act_i1 || r0 + ER - 2 * K <= s->act_i0 || c0 >= s->act_j1 || c0 + EC - 2 * K <= s->act_j0)
          continue;
        const int4 tile = make_int4(k, r0, c0, kind);
        if (q < nh) inner.push_back(tile);
        else if (q < ni) cold.push_back(tile);
        else pml.emplace_back(tile, planned);
      }
    }
    const int n_hot = (int)inner.size();
    inner.insert(inner.end(), cold.begin(), cold.end());
    // CPML tiles grouped by kind over every simulation (one kernel per kind), those with a plan
    // leading their kind
    std::stable_sort(pml.begin(), pml.end(), [](const std::pair<int4, bool>& p, const std::pair<int4, bool>& q) {
      return p.first.w != q.first.w ? p.first.w < q.first.w : p.second > q.second;
    });
    int n_kind[6] = {0, 0, 0, 0, 0, 0};
    for (const auto& q : pml) {
      n_kind[q.first.w - 1] += 1;
      n_kind[q.first.w + 2] += q.second;
    }
    const int n_inner = (int)inner.size(), n_pml = (int)pml.size();
    for (const auto& q : pml) inner.push_back(q.first);
    const bool same = b->d_tiles && n_inner == b->n_inner && n_pml == b->n_pml && n_hot == b->n_hot &&
                      memcmp(n_kind, b->n_kind, sizeof n_kind) == 0 && inner.size() == b->h_tiles.size() &&
                      memcmp(inner.data(), b->h_tiles.data(), inner.size() * sizeof(int4)) == 0;
    if (!same) {
      b->n_inner = n_inner;
      b->n_pml = n_pml;
      b->n_hot = n_hot;
      for (int k = 0; k < 6; ++k) b->n_kind[k] = n_kind[k];
      cudaFree(b->d_tiles);
      b->d_tiles = nullptr;
      int rc = etg_malloc((void**)&b->d_tiles, std::max<size_t>(1, inner.size()) * sizeof(int4));
      if (rc) return rc;
      ETG_TRY_CUDA(cudaMemcpy(b->d_tiles, inner.data(), inner.size() * sizeof(int4), cudaMemcpyHostToDevice));
      b->h_tiles.swap(inner);
      b->tiles_er = ER;
      b->tiles_k = K;
      *changed = true;
    }
  }
  return ETG_OK;
}

template <typename T>
int batch_advance(etg_batch* b, int64_t n_steps) {
  int ER, EC, K;
  tb_default_shape((int)sizeof(T), &ER, &EC, &K);
  if (b->opt[ETG_OPT_TILE_ROWS] > 0) ER = (int)b->opt[ETG_OPT_TILE_ROWS];
  if (b->opt[ETG_OPT_TB_DEPTH] > 0) K = (int)b->opt[ETG_OPT_TB_DEPTH];
  const int NW = b->opt[ETG_OPT_TB_WARPS] > 0 ? (int)b->opt[ETG_OPT_TB_WARPS] : 8;
  int rc = tb_batch_attrs<T>(ER, K, NW);
  if (rc) return rc;
  bool changed = false;
  rc = refresh<T>(b, ER, K, &changed);
  if (rc) return rc;
  if (changed) drop_graphs(b);
  const int n = (int)b->sims.size();
  const int64_t pairs = n_steps / (2 * K);
  const int64_t per_graph = std::max<int64_t>(1, b->opt[ETG_OPT_GRAPH_STEPS] / (2 * K));
  auto pair = [&](int64_t p) -> int {
    int r = tb_batch_pair<T>(ER, K, NW, b->d_sims, b->d_tiles, b->n_inner, b->n_hot, b->n_kind, 0, (int)(2 * K * p),
                             b->stream, b->sides, b->fork, b->joins);
    if (r == ETG_OK)
      r = tb_batch_pair<T>(ER, K, NW, b->d_sims, b->d_tiles, b->n_inner, b->n_hot, b->n_kind, 1, (int)(2 * K * p + K),
                           b->stream, b->sides, b->fork, b->joins);
    return r;
  };
  auto add_steps = [&](int64_t k) {
    k_batch_step_add<<<(n + 127) / 128, 128, 0, b->stream>>>(b->d_steps, n, k);
    g_launches += 1;
  };
  // a block: up to per_graph launch pairs, the DFT of the block's samples, the step counters
  auto block = [&](int64_t n_pairs) -> int {
    int r = ETG_OK;
    for (int64_t p = 0; p < n_pairs && r == ETG_OK; ++p) r = pair(p);
    if (r == ETG_OK) {
      tb_batch_dft<T>(b->d_sims, n, b->dft_work, b->dft_mon, (int)(2 * K * n_pairs), b->stream);
      add_steps(2 * K * n_pairs);
    }
    return r;
  };
  int64_t done = 0;
  if (b->opt[ETG_OPT_GRAPH_STEPS] > 0 && pairs >= per_graph) {
    auto it = b->graphs.find(per_graph);
    if (it == b->graphs.end()) {
      cudaGraph_t graph;
      ETG_TRY_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      const int r = block(per_graph);
      cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
      if (r) return r;
      ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
      cudaGraphExec_t exec;
      e = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      ETG_REQUIRE(e == cudaSuccess, ETG_ERR_CUDA, "batch graph instantiate failed: %s", cudaGetErrorString(e));
      it = b->graphs.emplace(per_graph, exec).first;
    }
    for (; done + per_graph <= pairs; done += per_graph) {
      ETG_TRY_CUDA(cudaGraphLaunch(it->second, b->stream));
      g_launches += 4 * per_graph + 2;
    }
  }
  while (done < pairs) {
    const int64_t c = std::min(per_graph, pairs - done);
    rc = block(c);
    if (rc) return rc;
    done += c;
  }
  const int64_t rem = n_steps - 2 * K * pairs;  // one-step kernels, simulation by simulation
  if (rem) {
    for (etg_sim* s : b->sims) {
      PhasePlan<T> ph, pe;
      rc = sim_plans_export<T>(s, &ph, &pe);
      if (rc) return rc;
      const SimArgs<T> a = sim_args_export<T>(s);
      for (int64_t k = 0; k < rem; ++k) launch_step_plain<T>(a, ph, pe, (int)k, b->stream);
    }
    add_steps(rem);
  }
  ETG_LAUNCH_CHECK();
  return ETG_OK;
}

}  // namespace

extern "C" {

int etg_batch_create(etg_batch** out, int n_sims, etg_sim* const* sims) {
  ETG_REQUIRE(out && sims && n_sims > 0, ETG_ERR_ARGUMENT, "etg_batch_create: bad arguments");
  for (int k = 0; k < n_sims; ++k) {
    ETG_REQUIRE(sims[k], ETG_ERR_ARGUMENT, "etg_batch_create: simulation %d is null", k);
    ETG_REQUIRE(sims[k]->dtype == sims[0]->dtype, ETG_ERR_ARGUMENT, "etg_batch_create: mixed precisions");
    ETG_REQUIRE(sims[k]->have_coeffs, ETG_ERR_STATE, "etg_batch_create: simulation %d has no coefficients", k);
    ETG_REQUIRE(!sims[k]->db_node, ETG_ERR_ARGUMENT,
                "etg_batch_create: simulation %d has per-node Hz coefficients (TM mode), which only the "
                "one-step kernels take; advance it on its own", k);
  }
  etg_batch* b = new etg_batch;
  b->sims.assign(sims, sims + n_sims);
  b->dtype = sims[0]->dtype;
  b->alt.assign(n_sims, nullptr);
  b->alt_bytes.assign(n_sims, 0);
  std::vector<int64_t*> steps(n_sims);
  for (int k = 0; k < n_sims; ++k) steps[k] = sims[k]->d_step;
  int rc = etg_malloc((void**)&b->d_steps, n_sims * sizeof(int64_t*));
  if (rc == ETG_OK &&
      (cudaMemcpy(b->d_steps, steps.data(), n_sims * sizeof(int64_t*), cudaMemcpyHostToDevice) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->sides[0], cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->sides[1], cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->sides[2], cudaStreamNonBlocking) != cudaSuccess ||
       cudaStreamCreateWithFlags(&b->sides[3], cudaStreamNonBlocking) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->joins[0], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->joins[1], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->joins[2], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreateWithFlags(&b->joins[3], cudaEventDisableTiming) != cudaSuccess ||
       cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess)) {
    set_error("etg_batch_create: %s", cudaGetErrorString(cudaGetLastError()));
    rc = ETG_ERR_CUDA;
  }
  if (rc) {
    etg_batch_destroy(b);
    return rc;
  }
  *out = b;
  return ETG_OK;
}

int etg_batch_destroy(etg_batch* b) {
  if (!b) return ETG_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (void* p : b->alt) cudaFree(p);
  cudaFree(b->d_sims);
  cudaFree(b->d_tiles);
  cudaFree(b->d_steps);
  for (cudaEvent_t e : {b->fork, b->join, b->ev0, b->ev1, b->done})
    if (e) cudaEventDestroy(e);
  if (b->side) cudaStreamDestroy(b->side);
  for (int k = 0; k < 4; ++k) {
    if (b->sides[k]) cudaStreamDestroy(b->sides[k]);
    if (b->joins[k]) cudaEventDestroy(b->joins[k]);
  }
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return ETG_OK;
}

int etg_batch_advance(etg_batch* b, int64_t n_steps) {
  ETG_REQUIRE(b && n_steps >= 0, ETG_ERR_ARGUMENT, "etg_batch_advance: bad arguments");
  if (fault_injected("etg_batch_advance")) return ETG_ERR_INJECTED;
  if (n_steps == 0) return ETG_OK;
  for (etg_sim* s : b->sims) {
    int rc = sim_check_tables(s, n_steps);
    if (rc) return rc;
    ETG_TRY_CUDA(cudaStreamSynchronize(s->stream));  // uploads on a simulation's own stream are done
  }
  const bool timing = b->opt[ETG_OPT_TIMING] != 0;
  const int64_t launches0 = g_launches;
  if (timing) ETG_TRY_CUDA(cudaEventRecord(b->ev0, b->stream));
  int rc = b->dtype == ETG_F32 ? batch_advance<float>(b, n_steps) : batch_advance<double>(b, n_steps);
  if (rc) return rc;
  if (timing) {
    ETG_TRY_CUDA(cudaEventRecord(b->ev1, b->stream));
    ETG_TRY_CUDA(cudaEventSynchronize(b->ev1));
    float ms = 0;
    ETG_TRY_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
  }
  b->last_launches = g_launches - launches0;
  // later work on a simulation's own stream (reads, uploads, single runs) waits for the batch
  ETG_TRY_CUDA(cudaEventRecord(b->done, b->stream));
  for (etg_sim* s : b->sims) {
    ETG_TRY_CUDA(cudaStreamWaitEvent(s->stream, b->done, 0));
    s->h_step += n_steps;
    s->psi_dirty = true;
  }
  return ETG_OK;
}

int etg_batch_synchronize(etg_batch* b) {
  ETG_REQUIRE(b, ETG_ERR_ARGUMENT, "etg_batch_synchronize: null handle");
  ETG_TRY_CUDA(cudaStreamSynchronize(b->stream));
  for (etg_sim* s : b->sims) {
    int rc = etg_sim_synchronize(s);
    if (rc) return rc;
  }
  return ETG_OK;
}

int etg_batch_set_option(etg_batch* b, int option, int64_t value) {
  ETG_REQUIRE(b && option >= 0 && option < 8 && value >= 0, ETG_ERR_ARGUMENT, "etg_batch_set_option: bad option");
  b->opt[option] = value;
  drop_graphs(b);
  return ETG_OK;
}

int etg_batch_last_timing(etg_batch* b, double* ms, int64_t* launches) {
  ETG_REQUIRE(b, ETG_ERR_ARGUMENT, "etg_batch_last_timing: null handle");
  if (ms) *ms = b->last_ms;
  if (launches) *launches = b->last_launches;
  return ETG_OK;
}

}  // extern "C"
