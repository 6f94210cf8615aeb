/* etalon_gb300 — C ABI of the GB300 (sm_103a) 2D TE FDTD backend for Etalon.
 *
 * Plain C types only: pointers, sizes, int status. Every entry point returns ETG_OK (0)
 * or an ETG_ERR_* code and leaves a message for etg_last_error() on the calling thread.
 * Arrays are C-ordered with y fastest, in the shapes of Etalon's TEState
 * (etalon/fdtd/state.py:15-49): Hz (nx, ny), Ex (nx, ny+1), Ey (nx+1, ny).
 * `dtype` is ETG_F32 or ETG_F64; complex arrays are interleaved (re, im) pairs.
 *
 * Paths in the comments are files of the Etalon project that each entry point
 * replaces or mirrors.
 */
#ifndef ETALON_GB300_H
#define ETALON_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define ETG_OK 0
#define ETG_ERR_ARGUMENT 1   /* bad size, pointer, id or dtype */
#define ETG_ERR_CUDA 2       /* a CUDA runtime call failed */
#define ETG_ERR_ALLOC 3      /* device or pinned allocation failed */
#define ETG_ERR_STATE 4      /* call not valid now (e.g. a table does not cover the steps) */
#define ETG_ERR_INJECTED 5   /* failure injected on the host (ETG_FAULT, tests only) */
#define ETG_ERR_NONFINITE 6  /* a field became NaN or Inf */
#define ETG_ERR_TIMEOUT 7    /* a bounded device-side wait gave up */

#define ETG_F32 4
#define ETG_F64 8

/* field ids (etalon/fdtd/state.py:15-49) */
#define ETG_EX 0
#define ETG_EY 1
#define ETG_HZ 2
#define ETG_PSI_EX_Y 3
#define ETG_PSI_EY_X 4
#define ETG_PSI_HZ_X 5
#define ETG_PSI_HZ_Y 6

/* ---------------------------------------------------------------- library */

/* Message of the last failed call on this thread ("" if none). */
const char* etg_last_error(void);
/* ABI version: (major << 16) | minor. */
int etg_version(void);
/* Current device ordinal, its name and SM count (replaces the device probe of
 * etalon/fdtd/backends/cupy_backend.py:36-59). */
int etg_device_info(int* device, char* name, int name_len, int* sm_count);
/* Wait for all work this library queued on the device. (cupy_backend.py:67-68) */
int etg_synchronize(void);
/* Make `device` current for this library on the calling thread (the library links its own
 * CUDA runtime, so the caller's current device does not carry over; cupy.cuda.Device). */
int etg_set_device(int device);

/* ---------------------------------------------------------------- device memory
 * Backing store of the per-step backend's device arrays
 * (replaces cupy.asarray / cupy.asnumpy in cupy_backend.py:61-65). */
int etg_malloc(void** ptr, size_t bytes);
int etg_free(void* ptr);
int etg_memcpy_h2d(void* dst, const void* src, size_t bytes);
int etg_memcpy_d2h(void* dst, const void* src, size_t bytes);
int etg_memcpy_d2d(void* dst, const void* src, size_t bytes);
int etg_memset(void* dst, int value, size_t bytes);
/* Page-locked host memory, for host<->device copies at full link speed. */
int etg_host_alloc(void** ptr, size_t bytes);
int etg_host_free(void* ptr);

/* ---------------------------------------------------------------- per-step protocol
 * One call = one backend method of Etalon's backend protocol
 * (etalon/fdtd/backends/__init__.py:1-53), on contiguous device arrays in TEState
 * layout. Results are bit-identical to NumpyBackend (IEEE order, no contraction). */

/* Hz^(n-1/2) -> Hz^(n+1/2) with CPML psi_hz_x/psi_hz_y.
 * Replaces update_te.cu:14-39 / numpy_backend.py:41-49. */
int etg_update_h_te(int dtype, int nx, int ny, void* hz, const void* ex, const void* ey,
                    void* psi_hz_x, void* psi_hz_y, const void* bx_h, const void* cx_h,
                    const void* ikx_h, const void* by_h, const void* cy_h, const void* iky_h,
                    double db, double inv_dx, double inv_dy);
/* Ex, Ey -> n+1 with CPML psi_ex_y/psi_ey_x; outer tangential E stays 0 (PEC).
 * Replaces update_te.cu:41-75 / numpy_backend.py:51-61. */
int etg_update_e_te(int dtype, int nx, int ny, void* ex, void* ey, const void* hz,
                    void* psi_ex_y, void* psi_ey_x, const void* cb_ex, const void* cb_ey,
                    const void* bx_e, const void* cx_e, const void* ikx_e, const void* by_e,
                    const void* cy_e, const void* iky_e, double inv_dx, double inv_dy);
/* acc[f, k] += field.flat[index[k]] * phasors[f]; acc (n_f, n_nodes) complex.
 * Replaces dft.cu:8-23 / numpy_backend.py:63-67. */
int etg_accumulate_dft(int dtype, int n_f, int n_nodes, void* acc, const void* field,
                       const int64_t* index, const void* phasors);
/* field[i[k], j[k]] -= delta[k] for k < n, field 2D with n_cols columns; NumPy
 * fancy-index semantics (all reads before writes, last duplicate wins).
 * Replaces the source injection of etalon/fdtd/solver.py:83-89. */
int etg_scatter_sub(int dtype, int64_t n_cols, int n, void* field, const int64_t* i,
                    const int64_t* j, const void* delta);

/* ---------------------------------------------------------------- reductions for the live view
 * Etalon Studio's progress energy and snapshot (etalon/studio/runner.py:258-291) on device
 * arrays, on the default stream like the per-step protocol. Rows of `pitch` elements. */
/* *out = sum over the rows x cols elements of f*f/c in float64 (c == NULL: f*f). */
int etg_sum_sq(int dtype, int64_t rows, int64_t cols, int64_t pitch, const void* field, const void* coeff,
               double* out);
/* out[(rows/sx) x (cols/sy)] (out_dtype, contiguous) = means of the sx x sy blocks, in float64. */
int etg_block_mean(int dtype, int64_t rows, int64_t cols, int64_t pitch, const void* field, int sx, int sy,
                   int out_dtype, void* out);
/* out[n] = in[n] converted between float32 and float64. */
int etg_cast(int from_dtype, int to_dtype, int64_t n, const void* in, void* out);

/* ---------------------------------------------------------------- fused simulation
 * A resident 2D TE run: fields, CPML strips, coefficients, per-step source deltas
 * and phasor tables all in HBM; etg_sim_advance runs whole steps (H, inject M,
 * DFT H, E, inject J, DFT E — etalon/fdtd/solver.py:120-128) with no host
 * round trip. Replaces FDTDSolver.step/run (solver.py:120-160). */
typedef struct etg_sim etg_sim;

/* 2 <= nx <= 262136 rows (x), 2 <= ny < 2^28 columns (y); larger grids are refused. */
int etg_sim_create(etg_sim** out, int dtype, int nx, int ny);
int etg_sim_destroy(etg_sim* sim);
/* Coefficients already cast to dtype (etalon/fdtd/state.py:75-97): cb_ex (nx, ny+1),
 * cb_ey (nx+1, ny), *_e of x (nx+1), *_h of x (nx), *_e of y (ny+1), *_h of y (ny). */
int etg_sim_set_coefficients(etg_sim* sim, const void* cb_ex, const void* cb_ey,
                             const void* bx_e, const void* cx_e, const void* ikx_e,
                             const void* bx_h, const void* cx_h, const void* ikx_h,
                             const void* by_e, const void* cy_e, const void* iky_e,
                             const void* by_h, const void* cy_h, const void* iky_h,
                             double db, double inv_dx, double inv_dy);
/* Replace a window of cb_ex (which = 0, array (nx, ny+1)) or cb_ey (which = 1, (nx+1, ny)):
 * rows [i0, i0+rows) x columns [j0, j0+cols) from a host array (rows, cols) in dtype. */
int etg_sim_set_cb_window(etg_sim* sim, int which, int i0, int rows, int j0, int cols, const void* host);
/* 2D TM mode (no counterpart in Etalon, which refuses TM: fdtd/capabilities.py:7-24). A TM run
 * (Ez, Hx, Hy) is stepped as its dual TE run: Ez in the Hz array, -Hx in Ex, -Hy in Ey, with
 * dt/mu0 as cb and dt/(eps0 eps_r) per Ez node in place of the scalar db. This uploads that
 * per-node coefficient, (nx, ny) in TEState Hz layout; from then on the simulation advances
 * with the one-step or the temporally blocked kernels (a TMA-fed kernel choice falls back to
 * the plain blocked one), and batches and the adjoint refuse it. */
int etg_sim_set_db_nodes(etg_sim* sim, const void* host);
/* cb_ex and cb_ey rasterised on the device from a staircase of boxes (etalon/grid/materials.py:12-35
 * with the cast of etalon/fdtd/state.py:80-81): node (i, j) of Ex sits at x = x_min + (i + 0.5) dx,
 * y = y_min + j dy, of Ey at x = x_min + i dx, y = y_min + (j + 0.5) dy; it takes eps of the last
 * box b with |x - cx| <= hx and |y - cy| <= hy (float64), else `background`; cb = dt / (eps0 eps)
 * in float64, cast to dtype. boxes: n_boxes rows of (cx, cy, hx, hy, eps), hx = sx/2 + tolerance
 * already added, boxes that miss the simulated plane already left out. Bit-identical to the host
 * rasterisation and cast; set the coefficients once first (the CPML profiles stay). Grids of at
 * most 65534 rows (nx). */
int etg_sim_rasterize_cb(etg_sim* sim, double x_min, double y_min, double dx, double dy, double dt,
                         double eps0, double background, int n_boxes, const double* boxes);
/* Copy cb_ex (which = 0, (nx, ny+1)) or cb_ey (which = 1, (nx+1, ny)) to a host array in dtype. */
int etg_sim_get_cb(etg_sim* sim, int which, void* host);
/* A point source on `component` (ETG_EX/EY/HZ) over n_nodes nodes (i, j) with its
 * per-step deltas for steps n0 .. n0+rows-1: table (rows, n_nodes) in dtype, the
 * values subtracted (etalon/fdtd/sources.py:54-56 cast to dtype). Sources apply in
 * the order they are added. */
int etg_sim_add_source(etg_sim* sim, int component, int n_nodes, const int64_t* i,
                       const int64_t* j, int64_t n0, int64_t rows, const void* table);
/* A DFT monitor component over the node rectangle [ix0, ix0+nxm) x [jy0, jy0+nym)
 * (x-major, etalon/fdtd/dft.py:92-107) at n_f frequencies, with phasor rows for steps
 * n0 .. n0+rows-1: table (rows, n_f) complex. Writes its id to *monitor. */
int etg_sim_add_monitor(etg_sim* sim, int component, int ix0, int nxm, int jy0, int nym,
                        int n_f, int64_t n0, int64_t rows, const void* table, int* monitor);
/* Replace the phasor rows of a monitor (next chunk of a long run). */
int etg_sim_set_phasors(etg_sim* sim, int monitor, int64_t n0, int64_t rows, const void* table);
/* Replace the delta rows of source number `source` (in order of addition). */
int etg_sim_set_deltas(etg_sim* sim, int source, int64_t n0, int64_t rows, const void* table);
/* Host <-> device copies of one field in TEState shape. */
int etg_sim_set_field(etg_sim* sim, int field, const void* host);
int etg_sim_get_field(etg_sim* sim, int field, void* host);
/* Device address and row pitch (elements) of one array of the simulation, for reading it in
 * place on the device (Etalon Studio's live view: etalon/studio/runner.py:258-291 reads
 * state.ex, ey, hz, cb_ex, cb_ey). array: 0-6 as the field ids, 7 = cb_ex, 8 = cb_ey. Element
 * (i, j) is at ptr + i * pitch + j; the address stays valid until the simulation is destroyed.
 * Reads must come after etg_sim_synchronize. */
int etg_sim_device_array(etg_sim* sim, int array, void** ptr, int64_t* pitch);
/* Accumulator of a monitor: (n_f, nxm*nym) complex. */
int etg_sim_get_dft(etg_sim* sim, int monitor, void* host);
int etg_sim_set_dft(etg_sim* sim, int monitor, const void* host);
/* Zero fields, psi and accumulators; step index back to 0. */
int etg_sim_reset(etg_sim* sim);
/* Run n_steps whole steps from the current step index. */
int etg_sim_advance(etg_sim* sim, int64_t n_steps);
int etg_sim_step_index(etg_sim* sim, int64_t* n);
int etg_sim_set_step_index(etg_sim* sim, int64_t n);
/* Block until the simulation's stream is idle; reports device-side errors. */
int etg_sim_synchronize(etg_sim* sim);
/* Tuning options (ETG_OPT_*), see below. */
int etg_sim_set_option(etg_sim* sim, int option, int64_t value);
int etg_sim_get_option(etg_sim* sim, int option, int64_t* value);
/* Device-side timing of the last etg_sim_advance (CUDA events on its stream):
 * total milliseconds and the number of kernel launches it made. */
int etg_sim_last_timing(etg_sim* sim, double* ms, int64_t* launches);
/* Per-kernel timing of the last advance run with ETG_OPT_TIMING = 2, which launches the
 * interior-tile and CPML-tile kernels of the temporally blocked path one after the other on
 * the simulation's stream, without graphs, with a CUDA-event pair around each launch, then
 * each kind of CPML tile once more on its own (same inputs, same outputs). Arrays of 5
 * (interior tiles without sources, monitors or traces; every other tile: CPML tiles and the
 * interior tiles with a source, monitor or trace node; CPML tiles across rows, across columns,
 * corners): total ms, launches, output cells inside the grid per launch. */
int etg_sim_kernel_timing(etg_sim* sim, double* ms, int64_t* launches, int64_t* cells);

/* ---------------------------------------------------------------- batch
 * No counterpart in Etalon (one FDTDSolver per simulation). Steps many resident simulations
 * of any sizes together, one launch pair per K steps for all of them; each keeps its own
 * tables, monitors and step index, and its result is bit-identical to its own run. The
 * simulations must share a precision; the batch does not own them. */
typedef struct etg_batch etg_batch;
int etg_batch_create(etg_batch** out, int n_sims, etg_sim* const* sims);
int etg_batch_destroy(etg_batch* batch);
/* Advance every simulation n_steps steps (asynchronous; etg_batch_synchronize waits). */
int etg_batch_advance(etg_batch* batch, int64_t n_steps);
int etg_batch_synchronize(etg_batch* batch);
/* ETG_OPT_TB_DEPTH, ETG_OPT_TILE_ROWS, ETG_OPT_GRAPH_STEPS, ETG_OPT_TIMING as for etg_sim. */
int etg_batch_set_option(etg_batch* batch, int option, int64_t value);
int etg_batch_last_timing(etg_batch* batch, double* ms, int64_t* launches);

/* ---------------------------------------------------------------- adjoint
 * No counterpart in Etalon. Gradient of an objective J(DFT accumulators) with respect to
 * cb_ex and cb_ey on a design window of cells [i0, i0+nxd) x [j0, j0+nyd): the Ex nodes
 * (i0..i0+nxd-1, j0..j0+nyd) and the Ey nodes (i0..i0+nxd, j0..j0+nyd-1). The window, with one
 * cell of margin, must lie where the CPML terms vanish, and hold no electric source. */
typedef struct etg_adj etg_adj;
int etg_adj_create(etg_adj** out, etg_sim* sim, int i0, int nxd, int j0, int nyd);
int etg_adj_destroy(etg_adj* adj);
/* Forward run of n_steps from zero fields (monitors accumulate as in etg_sim_advance).
 * stride 0 records Hz on the window at every step; stride S > 0 keeps a checkpoint every S
 * steps instead (fields and psi over the window's light cone for S steps) and recomputes each
 * segment, within that cone, in the backward pass. */
int etg_adj_forward(etg_adj* adj, int64_t n_steps, int64_t stride);
/* Reverse sweep: grad_acc[m] is dJ/d(accumulator m), (n_f, nodes) complex in dtype, or NULL
 * for monitors J does not use (one entry per monitor, in order of addition). Writes
 * dJ/dcb_ex (nxd, nyd+1) and dJ/dcb_ey (nxd+1, nyd) in float64. The simulation's fields are
 * left in an unspecified state. */
int etg_adj_backward(etg_adj* adj, const void* const* grad_acc, double* grad_cb_ex, double* grad_cb_ey);
/* The two halves of etg_adj_backward, for batches: set the objective's dJ/dacc (kept on the
 * device until replaced), and read dJ/dcb after a backward pass. */
int etg_adj_set_objective(etg_adj* adj, const void* const* grad_acc);
int etg_adj_gradient(etg_adj* adj, double* grad_cb_ex, double* grad_cb_ey);
/* Many designs at once (one adjoint context per simulation, one precision): the forward
 * passes step together as an etg_batch, and the reverse sweeps run as one set of K-step
 * launches over the tiles of every design. Each design's gradient is bit-identical to its
 * own etg_adj_backward. forward(n_steps, stride) as etg_adj_forward for every design; set
 * each design's objective, call backward, then read each gradient with etg_adj_gradient. */
typedef struct etg_adj_batch etg_adj_batch;
int etg_adj_batch_create(etg_adj_batch** out, int n, etg_adj* const* adjs);
int etg_adj_batch_destroy(etg_adj_batch* batch);
/* Options of the forward batch (ETG_OPT_TB_DEPTH, ETG_OPT_TILE_ROWS, ETG_OPT_GRAPH_STEPS). */
int etg_adj_batch_set_option(etg_adj_batch* batch, int option, int64_t value);
int etg_adj_batch_forward(etg_adj_batch* batch, int64_t n_steps, int64_t stride);
int etg_adj_batch_backward(etg_adj_batch* batch);

/* ---------------------------------------------------------------- no-allocation advance
 * Has no counterpart in Etalon. For callers that cannot allocate device memory when they
 * step fields: an application that owns all device memory through its own fixed arena, a
 * process under a hard device-memory budget, or a loop that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree. It advances fields the
 * caller owns by n_steps steps (no sources, no monitors) with the temporally blocked
 * kernel, and keeps its second buffer, tile list and step counter in one static device
 * array of ETG_STATIC_SCRATCH_BYTES, held by every GPU that loads the library until the
 * process exits. It calls no cudaMalloc, cudaFree or allocating library routine.
 *
 * Layout: every field, psi and cb array has nx + 2 rows of `pitch` elements (pitch a
 * multiple of 32 and >= ny + 1), element (i, j) at i * pitch + j, the TEState array in the
 * top-left corner and zeros elsewhere; pointers are 16-byte aligned. psi must be +0 wherever
 * the CPML c coefficient of its axis is 0 (true of any run started from zero fields).
 * 1D coefficients are contiguous as for etg_sim_set_coefficients.
 *
 * A grid needs 7 * (nx + 2) * pitch * dtype bytes plus its tile list; larger grids are
 * rejected with ETG_ERR_ARGUMENT. The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress, with that device current); make that first call before any
 * stream capture on that device.
 * Work runs on the default stream and the call returns when it is done. All calls share
 * the array and it keeps the last call's contents: calls that overlap on the GPU (from
 * several host threads) race. */
#define ETG_STATIC_SCRATCH_BYTES (16 << 20)
int etg_tb_advance_static(int dtype, int nx, int ny, int64_t pitch, void* ex, void* ey, void* hz,
                          void* psi_ex_y, void* psi_ey_x, void* psi_hz_x, void* psi_hz_y,
                          const void* cb_ex, const void* cb_ey, const void* bx_e,
                          const void* cx_e, const void* ikx_e, const void* bx_h, const void* cx_h,
                          const void* ikx_h, const void* by_e, const void* cy_e,
                          const void* iky_e, const void* by_h, const void* cy_h,
                          const void* iky_h, double db, double inv_dx, double inv_dy,
                          int64_t n_steps);

/* Test hook of the failure detection (no counterpart in Etalon): the iteration limit of the
 * first attempt of every bounded wait of the TMA-fed kernels (ETG_OPT_KERNEL 3 and 4) for
 * their shared-memory stage, on the current device. tries < 0 restores the default (2^20);
 * 0 gives up at once. A wait that runs out flags ETG_ERR_TIMEOUT (reported by the next
 * etg_sim_synchronize), waits once more, bounded, for the copy still in flight, and its CTA
 * returns. A limit of 0 makes real, completing copies time out, with no fault and no hang. */
int etg_debug_set_wait_tries(int64_t tries);

#define ETG_OPT_KERNEL 0        /* 0 = auto, 1 = one step per launch, 2 = temporal blocking,
                                   3 = temporal blocking, persistent CTAs fed by TMA (two per SM),
                                   4 = temporal blocking, one persistent CTA per SM claiming tiles,
                                       the next interior tile staged by TMA during the current one */
#define ETG_OPT_TB_DEPTH 1      /* steps per launch of the temporally blocked kernel */
#define ETG_OPT_GRAPH_STEPS 2   /* steps captured per CUDA graph (0 = no graphs) */
#define ETG_OPT_TILE_ROWS 3     /* tile rows of the temporally blocked kernel */
#define ETG_OPT_TILE_COLS 4     /* tile columns of the temporally blocked kernel */
#define ETG_OPT_CHECK_FINITE 5  /* 1 = flag NaN/Inf after each advance */
#define ETG_OPT_TB_WARPS 7      /* warps per CTA of the temporally blocked kernel (0: 8); the
                                   tile has TILE_ROWS / TB_WARPS rows per warp */
#define ETG_OPT_TIMING 6        /* 1 = record CUDA-event timing of each advance,
                                   2 = also time each temporally blocked kernel launch */
#define ETG_OPT_TB_SEGMENTS 8   /* 0 = lean interior tiles of one column stepped as segments by one
                                   CTA (a tile with its top halo, then three tiles that take the row
                                   above from their predecessor: five tiles' rows for four tiles'
                                   work, same bits) when the tile is 5K rows high and the segments
                                   at least fill the SMs; 1 = ordinary tiles only */
#define ETG_OPT_TB_SEGMENTS_USED 9  /* read-only: column segments of the current tile list */

/* ---------------------------------------------------------------- 3D Yee
 * Has no counterpart in Etalon: etalon/fdtd/capabilities.py:7-24 refuses 3D. The engine
 * carries Etalon's 2D TE discretisation to three axes (layout of etalon/grid/yee.py:27-79 with
 * a z axis, update order of etalon/fdtd/backends/numpy_backend.py:41-61 per component, step
 * order of etalon/fdtd/solver.py:83-128), so that a run invariant along a one-cell periodic
 * axis steps the other two exactly as the 2D TE update does.
 *
 * Arrays are C-ordered (x slowest, z fastest). Along a PEC axis of n cells a component has
 * n + 1 integer positions (both walls) or n half positions; along a periodic axis n of
 * either. Ex: (half, int, int), Ey: (int, half, int), Ez: (int, int, half), Hx: (int, half,
 * half), Hy: (half, int, half), Hz: (half, half, int). Tangential E on a PEC wall stays 0.
 *
 * Hx += db ((dEy/dz / kz + psi_hx_z) - (dEz/dy / ky + psi_hx_y)), Hy and Hz cyclically;
 * Ex += cb_ex ((dHz/dy / ky + psi_ex_y) - (dHy/dz / kz + psi_ex_z)),
 * Ey -= cb_ey ((dHz/dx / kx + psi_ey_x) - (dHx/dz / kz + psi_ey_z)),
 * Ez += cb_ez ((dHy/dx / kx + psi_ez_x) - (dHx/dy / ky + psi_ez_y)),
 * psi <- b psi + c d before each use; one IEEE rounding per operation, no fused multiply-add.
 * A step is H, H sources, H monitors, E, E sources, E monitors (etg_yee3d_set_option). */
#define ETG3_EX 0
#define ETG3_EY 1
#define ETG3_EZ 2
#define ETG3_HX 3
#define ETG3_HY 4
#define ETG3_HZ 5
/* array ids 6..17: psi_hx_y psi_hx_z psi_hy_z psi_hy_x psi_hz_x psi_hz_y psi_ex_y psi_ex_z
 * psi_ey_z psi_ey_x psi_ez_x psi_ez_y (each shaped as its field); 18..20: cb_ex cb_ey cb_ez */
#define ETG3_PSI0 6
#define ETG3_CB0 18
typedef struct etg_yee3d etg_yee3d;
/* periodic_mask: bit a set = axis a (0 x, 1 y, 2 z) periodic. Fields, psi and cb start at 0;
 * profiles start as b = 1, c = 0, 1/kappa = 1 (no CPML). Grids need nx < 65535, ny < 458738
 * and (ny + 1) * Pz < 2^31 with Pz = nz + 1 rounded up to 8; larger ones are refused. */
int etg_yee3d_create(etg_yee3d** out, int dtype, int nx, int ny, int nz, int periodic_mask);
int etg_yee3d_destroy(etg_yee3d* sim);
/* db, 1/dx, 1/dy, 1/dz (1/m), four values of the run's dtype */
int etg_yee3d_set_scalars(etg_yee3d* sim, const void* host4);
/* CPML profile of one axis: b, c, 1/kappa at the integer positions (n + 1 on a PEC axis, n on
 * a periodic one) and at the n half positions (etalon/fdtd/cpml.py:74-92 per axis). psi is
 * kept only where b != 1 or c != 0: leading and trailing strips of each profile. */
int etg_yee3d_set_profile(etg_yee3d* sim, int axis, const void* b_e, const void* c_e, const void* ik_e,
                          const void* b_h, const void* c_h, const void* ik_h);
/* whole arrays, C-ordered in the shapes above; psi must be +0 outside the strips, and the
 * psi of an axis without CPML is not stored (set accepts only zeros, get returns zeros) */
int etg_yee3d_set_field(etg_yee3d* sim, int array, const void* host);
int etg_yee3d_get_field(etg_yee3d* sim, int array, void* host);
/* field[nodes] -= table[n - n0] at step n, nodes as flat C-order indices into the component
 * (at most 64; etalon/fdtd/solver.py:83-89); table: rows x n_nodes of the dtype */
int etg_yee3d_add_source(etg_yee3d* sim, int component, int n_nodes, const int64_t* flat, int64_t n0,
                         int64_t rows, const void* table);
/* acc[f, node] += field[node] * phasor[n - n0, f] (etalon/fdtd/backends/numpy_backend.py:63-67);
 * table: rows x n_f complex of the dtype; accumulators start at 0 */
int etg_yee3d_add_monitor(etg_yee3d* sim, int component, int n_nodes, const int64_t* flat, int n_f,
                          int64_t n0, int64_t rows, const void* table);
int etg_yee3d_get_dft(etg_yee3d* sim, int monitor, void* host);
/* n_steps steps on the engine's stream (asynchronous); ETG_ERR_STATE if a table does not
 * cover them */
int etg_yee3d_advance(etg_yee3d* sim, int64_t n_steps);
int etg_yee3d_synchronize(etg_yee3d* sim);
int etg_yee3d_step_index(etg_yee3d* sim, int64_t* n);
/* device time (CUDA events) of the last etg_yee3d_advance and its kernel launches */
int etg_yee3d_last_timing(etg_yee3d* sim, double* ms, int64_t* launches);
/* n_steps more steps, each stencil launch timed alone: mean ms per launch of the fused step's
 * kernel (ms_h; ms_e = 0) or of the H and E kernels of the two-kernel step */
int etg_yee3d_kernel_timing(etg_yee3d* sim, int n_steps, double* ms_h, double* ms_e);
/* ETG3_OPT_FUSED (default 0): 0 = an H and an E kernel per step, in place, sources by their
 * own kernels; 1 = one kernel per step, H and E together, from one buffer set into a second
 * (allocated at the first such step: twice the field and psi memory), point sources applied
 * inside it (at most 16 per phase, 32 distinct nodes per phase; more run the two-kernel step).
 * Both give the same bits; the two-kernel step is the faster on GB300. */
#define ETG3_OPT_FUSED 0
int etg_yee3d_set_option(etg_yee3d* sim, int option, int64_t value);

#ifdef __cplusplus
}
#endif
#endif /* ETALON_GB300_H */
