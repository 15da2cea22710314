/*
 * rift_gb300.h -- C ABI of the GB300-native RIFT shallow-water step.
 *
 * The reference drives its device step through the C++ launcher set in
 * grid.h:6-63 (SetDeviceConstants, AllocateGrid, InitGrid, ComputeFluxes,
 * Integrate_1, Integrate_2, Grow, ApplyBoundaries, InterpGrid, FillGrid,
 * SumReduce, FreeGrid) plus the dt reduction in simulator.cu:540-566
 * (Simulator::ComputeTimestep) and the source hooks simulator.cu:891-907.
 * Those launchers take raw FP64 pitched device pointers and keep their state
 * in __constant__ symbols and host globals.  This header replaces that seam
 * with an opaque handle: the handle owns every device buffer, one CUDA
 * stream per handle, every call returns an int status (never exit()).
 *
 * Host arrays exchanged through this ABI use the reference's host layout:
 * row-major FP64, h_ny rows of h_nx cells (the 2-cell ghost ring included),
 * cell (j,i) at [j*ld + i].  BX is h_ny x (h_nx+1) (west face of cell i at
 * column i), BY is (h_ny+1) x h_nx (south face of cell j at row j), as built
 * by Simulator::InitSimulation (simulator.cu:384-431).
 *
 * Tiles are the reference's 16 x 14 cell blocks (grid.cu:18-19):
 * nBX = ceil(h_nx/16), nBY = ceil(h_ny/14), tile id = bY*nBX + bX.
 */
#ifndef RIFT_GB300_H
#define RIFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define RIFT_OK            0
#define RIFT_ERR_ARG       1  /* bad argument (null pointer, bad size, bad enum) */
#define RIFT_ERR_CUDA      2  /* a CUDA runtime call failed; see rift_last_error */
#define RIFT_ERR_STATE     3  /* call out of order (e.g. step before init) */
#define RIFT_ERR_NUMERIC   4  /* device detected a non-finite or negative depth */
#define RIFT_ERR_NOMEM     5  /* device allocation failed */
#define RIFT_ERR_UNSUPPORTED 6

/* ---- feature flags: the reference's __constant__ bools (grid.cu:21-25) -- */
#define RIFT_F_RAIN_UNIFORM  (1u << 0)  /* rainfall_averaged: hyetograph CSV */
#define RIFT_F_RAIN_GRID     (1u << 1)  /* rainfall_gridded: rain map series */
#define RIFT_F_DRAIN_UNIFORM (1u << 2)  /* drain_averaged */
#define RIFT_F_DRAIN_GRID    (1u << 3)  /* drain_gridded */
#define RIFT_F_INFILTRATION  (1u << 4)  /* Green-Ampt (K, psi, dtheta) */
#define RIFT_F_SURGE_GRID    (1u << 5)  /* surge_gridded */
#define RIFT_F_EULER         (1u << 6)  /* euler_integration: stage 1 only */
#define RIFT_F_SAVE_MAX      (1u << 7)  /* h_max, q_max (+ t_peak, t_dry in Euler mode) */
#define RIFT_F_SAVE_ARRIVAL  (1u << 8)  /* t_wet */
#define RIFT_F_TILE_ACCEL    (1u << 9)  /* tile_acceleration: skip dry tiles */
#define RIFT_F_POINT_SOURCE  (1u << 10) /* dambreak: hydrograph point/rect source */
#define RIFT_F_H_INIT        (1u << 11) /* h_init: initial depth map */
#define RIFT_F_CHECK_VOLUME  (1u << 12) /* check_volume: keep the full volume ledger */

/* ---- map slots for rift_set_map ---------------------------------------- */
#define RIFT_MAP_RAIN  0  /* m/s, hyetograph_gridded_rate */
#define RIFT_MAP_DRAIN 1  /* m/s, drain_gridded_rate */
#define RIFT_MAP_SURGE 2  /* m,   surge_gridded_depth (nodata aware) */

/* ---- field ids for rift_get_field -------------------------------------- */
#define RIFT_FIELD_W     0   /* water-surface elevation (FP64, ghost ring included) */
#define RIFT_FIELD_HU    1
#define RIFT_FIELD_HV    2
#define RIFT_FIELD_F     3   /* Green-Ampt cumulative infiltration */
#define RIFT_FIELD_H     4   /* clamped depth map (dev_h, Integrate_2_k:1108-1111) */
#define RIFT_FIELD_Q     5   /* unit discharge map (dev_q, Integrate_2_k:1113-1119) */
#define RIFT_FIELD_HMAX  6
#define RIFT_FIELD_QMAX  7
#define RIFT_FIELD_TPEAK 8
#define RIFT_FIELD_TDRY  9
#define RIFT_FIELD_TWET  10
#define RIFT_FIELD_BC    11  /* cell-centre bed elevation (InitGrid_k:532) */

typedef struct rift_grid_desc {
    int32_t  h_nx, h_ny;   /* cells incl. ghost ring; b_nx+3 (grid_config.cpp:84-85) */
    double   dx, dy;       /* h_dx, h_dy in metres */
    double   kappa;        /* desingularisation constant (simulator.cu:281) */
    double   nodata;       /* GridConfig::nodata (-9999) */
    double   courant;      /* courant_max (simulator.cu:61-72) */
    double   psi, dtheta;  /* Green-Ampt suction head and moisture deficit */
    uint32_t flags;        /* RIFT_F_* */
    int32_t  device;       /* CUDA device ordinal */
} rift_grid_desc;

typedef struct rift_handle rift_handle;

/* Replaces SetDeviceConstants (grid.cu:321) + AllocateGrid (grid.cu:347). */
int rift_create(const rift_grid_desc* g, rift_handle** out);

/* Replaces the H2D uploads of simulator.cu:433-450.  n and K are per-cell
 * (h_ny x h_nx); K is already in m/s (simulator.cu:426).  h0 may be NULL. */
int rift_upload_static(rift_handle* h, const double* BX, const double* BY,
                       const double* n, const double* K_mps, const double* h0);

/* Replaces InitGrid (grid.cu:556) followed by ApplyBoundaries (simulator.cu:731).
 * Sets t = t0, dt_prev = 1e-7f (simulator.cu:35). */
int rift_init(rift_handle* h, double t0);

/* Uniform rain and drain rates for the next rift_step, m/s (the caller's
 * Source::interpolated_rate after unit conversion, simulator.cu:500-538). */
int rift_set_uniform_rates(rift_handle* h, double rain_mps, double drain_mps);

/* Point / rectangular hydrograph source cells: flat indices j*h_nx+i and
 * rates in m/s (Simulator::InitializeSources/setSourceValue,
 * simulator.cu:858-907). */
int rift_set_point_sources(rift_handle* h, const int32_t* idx,
                           const double* rate_mps, int32_t n);

/* New rates (m/s per source cell) for the n cells of the last
 * rift_set_point_sources call, used from the next step on: the device copy of
 * Simulator::updateSources (simulator.cu:903-907).  The source cells, the
 * per-tile source lists and the captured step graph are kept.  A hydrograph
 * series (rift_set_series which = 2) replaces them at the start of each step,
 * as UpdateSource does in the reference (simulator.cu:502-518).
 * RIFT_ERR_ARG when n differs from the source count. */
int rift_set_point_rates(rift_handle* h, const double* rate_mps, int32_t n);

/* Gridded map for the next step (GridSeries::update, GridSeries.cu:144-403).
 * t1map == NULL: hold t0map.  Otherwise the map is
 * InterpGrid(factor, t0map, t1map) (grid.cu:292-311), evaluated on device. */
int rift_set_map(rift_handle* h, int32_t which, const double* t0map,
                 const double* t1map, double factor);

/* Only the interpolation factor changes (same t0/t1 maps). */
int rift_set_map_factor(rift_handle* h, int32_t which, double factor);

/* The interpolation factor of map `which` follows the simulated time:
 * factor = (t - t0) / (t1 - t0) at the start of every step, the value
 * InterpolatedGridSeries::p_update computes after the previous step
 * (GridSeries.cu:398).  t1 <= t0 turns it off (fixed factor). */
int rift_set_map_times(rift_handle* h, int32_t which, double t0, double t1);

/* One full RK2 (or Euler) step, Grow included: the body of
 * Simulator::RunSimulation (simulator.cu:773-853) from Grow to the last
 * ApplyBoundaries.  Returns the new t and dt. */
int rift_step(rift_handle* h, double* t, double* dt);

/* Run nsteps steps on device without a host round trip per step: one
 * persistent cooperative launch while few tiles are active, else per-step
 * CUDA graph replays.  Uniform rates / maps stay as last set.  Stops early
 * once t >= t_stop. */
int rift_run(rift_handle* h, int32_t nsteps, double t_stop, double* t,
             double* dt, int32_t* steps_done);

/* Device-resident uniform CSV series (Source::InterpolateRate,
 * source.cc:65-73, with the in-place unit division of simulator.cu:500-538).
 * which: 0 = hyetograph (mm/hr), 1 = drain (mm/hr), 2 = hydrograph (cfs,
 * spread over the point-source cells).  times in seconds. */
int rift_set_series(rift_handle* h, int32_t which, const float* times_s,
                    const float* rates, int32_t n);

/* Copy a field to host memory, h_ny rows with leading dimension ld. */
int rift_get_field(rift_handle* h, int32_t which, double* host, size_t ld);

/* Tile state in the reference encoding: wet flag per tile (GridSize bytes),
 * the active tile ids sorted ascending, and their count. */
int rift_get_tiles(rift_handle* h, uint8_t* wet, int32_t* active,
                   int32_t* n_active);

/* Per-tile local speed maxima mx/my (GridSize doubles each). */
int rift_get_tile_speeds(rift_handle* h, double* mx, double* my);

/* Hotstart-style state upload (Simulator::ReadHotstart, simulator.cu:975).
 * active_ids (sorted ids of the active tiles, n_active of them), F, wet, mx
 * and my may be NULL (n_active < 0 keeps the current active set). */
int rift_set_state(rift_handle* h, double t, double dt_prev, const double* w,
                   const double* hu, const double* hv, const double* F,
                   const uint8_t* wet, const int32_t* active_ids,
                   int32_t n_active, const double* mx, const double* my);

/* Current t and dt. */
int rift_get_time(rift_handle* h, double* t, double* dt);

/* FP64 compensated volume sum over interior cells of (h [+F]), m of depth
 * summed (multiply by dx*dy for m^3) -- the device counterpart of the host
 * volume check in simulator.cu:609-637. */
int rift_volume(rift_handle* h, double* volume);

/* Volume ledger (replaces the check_volume accounting of
 * Simulator::UpdateSource / setSourceValue / RunSimulation,
 * simulator.cu:524-530, 819-820, 892-897): `volume` as rift_volume, `added`
 * the FP64 sum since rift_init of the volume (depth x cells) the sources
 * applied -- per step, dt x (uniform rain rate x interior cells + point
 * source rates + interior sum of the gridded rain map at the step's
 * factor).  The reference adds uniform rain with the previous step's dt;
 * this ledger uses the dt the step applied, so that with no outflow,
 * drain, infiltration or clamping, volume - volume(init) = added up to the
 * FP32 rounding of the state. */
int rift_mass_ledger(rift_handle* h, double* volume, double* added);

/* The full FP64 volume ledger (the check_volume accounting of
 * simulator.cu:524-530, 609-637, 819-820, 892-897, completed with every way
 * the step adds or removes water: the clamps of grid.cu:748-749, 914-915,
 * 1083-1084, the drain and infiltration caps of grid.cu:776-805, the surge
 * condition of grid.cu:894-904 and the critical-depth ghosts of
 * grid.cu:1325-1406).  Depths summed over interior cells (times dx*dy for
 * m^3), since the ledger's start (rift_init or rift_set_state):
 *   volume - volume0 = added - drained - infiltrated - clamped + surge + boundary
 * and, with infiltration, soil - soil0 = infiltrated.  Each term is the
 * state change it caused: an RK2 step applies half of each stage's rates for
 * dt (Euler: the single stage's), and the clamps' removals as applied.  The
 * terms after `added`, and volume0 / soil0, are kept only when the handle
 * was created with RIFT_F_CHECK_VOLUME (a few operations per cell and
 * stage); otherwise they read 0 (volume0, soil0: NaN).  The ensemble kernel
 * does not keep them (rift_ensemble_create rejects such members). */
typedef struct rift_ledger {
    double volume, soil;       /* sums of h and of F (Green-Ampt) now */
    double volume0, soil0;     /* the same at the ledger's start */
    double added;              /* uniform rain, gridded rain and point sources */
    double drained;            /* uniform and gridded drain, after the h/dt cap */
    double infiltrated;        /* Green-Ampt rates, after the h/dt cap */
    double clamped;            /* depth the epsilon clamps removed (net) */
    double surge;              /* depth the surge condition added (net) */
    double boundary;           /* net inflow through the domain edge */
} rift_ledger;
int rift_mass_ledger_terms(rift_handle* h, rift_ledger* out);

/* Measurement entry point (no reference counterpart; the reference only
 * prints a wall-clock Mcells/s line, simulator.cu:836-841): nsteps step-graph
 * replays timed with CUDA events on the handle's stream (ms_total; summed
 * active interior cells in active_total; steps_done), then up to 20 more
 * steps launched one by one with events around the two fused stage kernels
 * (stage_ms = their mean duration per step, active_cells = mean active
 * interior cells per step of that pass). */
int rift_bench_run(rift_handle* h, int32_t nsteps, double* ms_total,
                   double* active_total, double* steps_done, double* stage_ms,
                   double* active_cells);

/* Kernel schedule (no reference counterpart; the reference launches one CTA
 * per active tile): from march_min_strips active strips of 7 x 2 tiles
 * upward the step runs the column-march kernels, below it the per-tile
 * kernels.  Both give the same results.  -1 restores the default (one strip
 * per resident march CTA); 0 forces the march, a huge value the tiles. */
int rift_set_schedule(rift_handle* h, int32_t march_min_strips);

/* Persistent step loop (no reference counterpart): while at most
 * max_active_tiles tiles are active, rift_run / rift_step run their steps
 * in one cooperative launch whose phases are separated by grid barriers,
 * with the per-tile arithmetic of the per-step kernels.  -1 restores the
 * default (the march threshold in tiles), 0 turns it off.
 * RIFT_ERR_UNSUPPORTED when the device has no cooperative launch. */
int rift_set_persistent(rift_handle* h, int32_t max_active_tiles);

/* Height of the column march's work items (no reference counterpart): 1, 2
 * (default) or 4 reference tile rows, i.e. CTA items of 112 x 14, 112 x 28
 * or 112 x 56 cells.  Each item stages its rows with a 2-row halo, so taller
 * items stage fewer rows twice and shorter ones balance a ragged active set
 * better.  The activity tiles stay 16 x 14: every height gives the same
 * results. */
int rift_set_march_rows(rift_handle* h, int32_t tile_rows);
int rift_get_march_rows(rift_handle* h, int32_t* tile_rows);

/* Autotuner of the schedule and the march's work-item shape (no reference
 * counterpart): from the current state, runs probe_steps steps on each
 * candidate -- 0 the persistent loop, 1 the per-step graph with the per-tile
 * kernels (one 16 x 14 tile per CTA of 256 threads), 2, 3, 4 the graph with
 * the column-march kernels on items of 2, 1 and 4 tile rows (128 threads per
 * 7-tile-wide item) -- timing each with CUDA events, restores the state
 * exactly, and keeps the fastest (as rift_set_persistent / rift_set_schedule
 * / rift_set_march_rows would set it).  choice: the candidate's index;
 * ms_per_step[RIFT_AUTOTUNE_CANDIDATES] (may be NULL): the measured times
 * (NaN for a candidate not available). */
#define RIFT_AUTOTUNE_CANDIDATES 5
int rift_autotune(rift_handle* h, int32_t probe_steps, int32_t* choice, double* ms_per_step);

/* Ensembles (no reference counterpart; the reference runs one scenario per
 * process): members -- handles created, uploaded and initialised as usual,
 * on one device, of any sizes and options -- advance together in one
 * persistent cooperative kernel that walks device queues of (member, tile)
 * work items; each member keeps its own dt, t, sources and outputs, and its
 * results are those of a run of its own.  rift_ensemble_run advances each
 * member until t >= t_stop or max_steps of its steps; t_out and steps_out
 * (n entries each, may be NULL) receive each member's final t and steps.
 * The members must not be stepped elsewhere while an ensemble runs them. */
typedef struct rift_ensemble rift_ensemble;
int rift_ensemble_create(rift_handle* const* members, int32_t n, rift_ensemble** out);
int rift_ensemble_run(rift_ensemble* e, double t_stop, int32_t max_steps, double* t_out,
                      int32_t* steps_out);
/* Members with at least min_cells interior cells (0, the default: none) are
 * not stepped by the persistent ensemble kernel: after it, each of them runs
 * on its own per-step graph, smallest first, with the whole GPU (the column
 * march on dense grids, about 2.5x the cell rate of the kernel's per-tile
 * code).  Their results are those of a run of their own, as every member's. */
int rift_ensemble_set_solo_cells(rift_ensemble* e, int64_t min_cells);
/* Per member (n entries): the device time, in seconds, from the start of the
 * last rift_ensemble_run's kernel to the end of the member's last step in it
 * (the GPU's global timer, read when the member's final iteration ends; for
 * members run on their own, CUDA events, counted after the kernel and the
 * members run before them); 0 for a member that ran no step. */
int rift_ensemble_member_times(rift_ensemble* e, double* seconds);
/* Kernels launched so far by rift_ensemble_run: its ensemble kernels plus
 * the launches of the members run on their own (rift_get_launch_count). */
int rift_ensemble_launch_count(rift_ensemble* e, int64_t* kernels);
const char* rift_ensemble_last_error(rift_ensemble* e);
void rift_ensemble_destroy(rift_ensemble* e);

/* Steps run so far by the persistent launch and by the per-step graph. */
int rift_get_path_stats(rift_handle* h, int64_t* persist_steps, int64_t* graph_steps);

/* Kernels launched so far by rift_run / rift_step on this handle: each
 * persistent launch counts one, each replay of the per-step graph the
 * kernels in it. */
int rift_get_launch_count(rift_handle* h, int64_t* kernels);

/* Of the persistent steps, those run from the loop's tile table: one
   scheduled tile per CTA kept from step to step, no grow phase (no gridded
   rain or surge, RK2).  No reference counterpart. */
int rift_get_table_steps(rift_handle* h, int64_t* table_steps);

/* Sizes: GridSize (tiles) and the tile grid. */
int rift_get_tile_grid(rift_handle* h, int32_t* nBX, int32_t* nBY);

/* Host-array access path (no reference counterpart).  Where the device
 * reads and writes pageable host memory through the host's page tables
 * (Grace + GB300 over NVLink-C2C: cudaDevAttrPageableMemoryAccess and
 * ...UsesHostPageTables both 1), rift_set_state converts the caller's FP64
 * arrays on the device, reading them in place, and rift_get_field writes the
 * FP64 field straight into the caller's array; the results are bit for bit
 * those of the staged host path.  Off by default: on GB300 it measured
 * slower than the staged copies (config 2: 11 ms against 5 ms for one
 * upload and one depth readback of 2048^2 cells).  rift_set_host_access(h, 1)
 * turns it on (RIFT_ERR_UNSUPPORTED where the device cannot), (h, 0) off. */
int rift_set_host_access(rift_handle* h, int32_t on);
int rift_get_host_access(rift_handle* h, int32_t* on);

/* Device-side view of a handle's state, for kernels of other libraries that
 * run between steps on the handle's stream (the learned flux closure).  No
 * reference counterpart.  Every plane is FP32 with `pitch` floats per row and
 * `rows` rows; cell (j, i) of the h-grid (ghost ring included) sits at
 * [j*pitch + i].  h, hu, hv hold U^n between calls; e holds four planes one
 * plane (rows*pitch floats) apart: eW, eE, eS, eN, each face elevation minus
 * the cell's reference elevation.  t and dt point at the device FP64
 * simulated time and the last step's dt, valid once the previous call has
 * returned.  A caller may change h, hu and hv of interior cells that are not
 * next to the ghost ring (3 <= i <= h_nx-4, 3 <= j <= h_ny-4) between calls,
 * on `stream`, provided no wet cell (h > 1.19e-7 m) becomes dry and no dry
 * cell wet: the tile activity the engine tracks then stays exact. */
typedef struct rift_device_view {
    float* h;
    float* hu;
    float* hv;
    const float* e;
    const float* n;
    const double* t;
    const double* dt;
    void* stream;        /* cudaStream_t */
    int32_t h_nx, h_ny, pitch, rows;
    double dx, dy, kappa;
} rift_device_view;
int rift_get_device_view(rift_handle* h, rift_device_view* v);

/* Volume sum for callers that cannot allocate device memory.  This entry
 * point has no counterpart in the reference.
 *
 * Some callers must not call cudaMalloc: a coupled model (for instance the
 * 1D drainage side of a 1D-2D coupling) that checks the 2D mass balance from
 * inside its own time loop, whose device memory comes from its own pool, or
 * that is recording work on a stream it does not want synchronised --
 * cudaMalloc and cudaFree synchronise the whole device.  This call takes
 * only the caller's buffers and allocates nothing: its scratch (one FP64
 * compensated partial sum per grid row) is a fixed array inside this
 * library's device image, present on every GPU that loads the library until
 * the process exits.
 *
 * depth: device pointer to an FP32 depth field, h_ny rows with leading
 *        dimension ld floats, cell (j,i) at depth[j*ld + i]; only interior
 *        cells (2 <= i,j <= n-3) are summed;
 * infil: optional device pointer to the Green-Ampt F field, same layout;
 * volume_dev: device pointer to one double receiving sum(h [+ F]) (metres of
 *        depth summed; multiply by dx*dy for m^3);
 * stream: the cudaStream_t to launch on (NULL: the legacy default stream).
 * The call is asynchronous on `stream`.
 * Limits: h_ny <= RIFT_NOALLOC_MAX_ROWS, else RIFT_ERR_TOO_LARGE and nothing
 * is launched.  All calls on a device share the scratch array, which keeps
 * the last call's partial sums (each call rewrites every partial it reads);
 * calls that overlap on the GPU race on it and must be serialised by the
 * caller.  The first call on each device looks up the array's address with
 * that device current; make it before recording any stream capture there.
 * The address is remembered with the id of the context it was found in: the
 * first call after a cudaDeviceReset (a new primary context) looks it up
 * again, so make that call outside stream capture too. */
#define RIFT_NOALLOC_MAX_ROWS 32768
#define RIFT_ERR_TOO_LARGE 7
int rift_volume_noalloc(const float* depth, const float* infil, int32_t h_nx,
                        int32_t h_ny, int64_t ld, double* volume_dev,
                        void* stream);

const char* rift_last_error(rift_handle* h);
void rift_destroy(rift_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* RIFT_GB300_H */
