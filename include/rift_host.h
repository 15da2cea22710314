/*
 * rift_host.h -- C ABI of the host drop-in layer above the GB300 step
 * (include/rift_gb300.h): the reference's file formats and its Simulator
 * life cycle.
 *
 * Replaces, on the reference side:
 *   ConfigFile (config.h:45-209)                   -> rift_config_*
 *   InitBathymetry / ReadGrid / SetOriginalGrid /
 *     writeGrid (io.cc:28-361)                     -> rift_esri_*
 *   GridConfig (grid_config.cpp:67-170)            -> rift_gridconfig_*
 *   Source::ReadSource / InterpolateRate
 *     (source.cc:11-73)                            -> rift_csv_read
 *   Simulator::WriteHotstart / ReadHotstart
 *     (simulator.cu:912-1090)                      -> rift_hotstart_*
 *   Simulator::OpenSimulation / RunSimulation /
 *     CloseSimulation (simulator.cu:711-853)       -> rift_sim_*
 *
 * Every function returns RIFT_OK (0) or an RIFT_ERR_* code of
 * rift_gb300.h; none exits or reads standard input (the reference's
 * ConfigFile waits on stdin and exits on a bad line).  Messages of the
 * last failure: rift_host_last_error() (per thread) or
 * rift_sim_last_error().
 */
#ifndef RIFT_HOST_H
#define RIFT_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "rift_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* GridConfig (grid_config.hpp:15-40): corner raster (b_*) and h-grid
 * (h_*, ghost ring of 2 included; h_nx = b_nx + 3). */
typedef struct rift_gridconfig {
    int32_t b_nx, b_ny;
    double b_xll, b_yll, cellsize_original;
    int32_t h_nx, h_ny;
    double h_xll, h_yll, cellsize, h_dx, h_dy;
    uint8_t square_cells, projected;
} rift_gridconfig;

const char* rift_host_last_error(void);

/* ---- keyword = value configuration (config.h) -------------------------
 * Lines: text after ';' is a comment; blank lines are skipped; a line needs
 * '=' with a non-blank value; the key ends at the first blank; duplicate
 * keys are an error. */
typedef struct rift_config rift_config;
int rift_config_open(const char* path, rift_config** out);
int rift_config_has(const rift_config* c, const char* key);
/* value as written (trimmed); RIFT_ERR_ARG if the key is absent */
int rift_config_get(const rift_config* c, const char* key, char* buf, size_t cap);
/* the reference's keyIsNumber: non-empty and only digits and '.' */
int rift_config_is_number(const rift_config* c, const char* key);
int rift_config_get_double(const rift_config* c, const char* key, double* v);
void rift_config_close(rift_config* c);

/* ---- ESRI ASCII rasters (io.cc) ---------------------------------------- */
int rift_esri_read_header(const char* path, int32_t* ncols, int32_t* nrows, double* xll,
                          double* yll, double* cellsize, double* nodata);
/* values into out[nrows][ncols] with row 0 the SOUTH row (the file's last
 * line), as the reference stores them; a NODATA value is an error unless
 * nodata_ok, when it becomes -9999 (GridConfig::nodata) */
int rift_esri_read(const char* path, int32_t ncols, int32_t nrows, int32_t nodata_ok,
                   double* out);
/* writeGrid: the interior of an h-grid array x[h_ny][h_nx], north row
 * first, 15 significant digits, header from gc */
int rift_esri_write_hgrid(const char* path, const double* x, const rift_gridconfig* gc);

/* GridConfig of a corner DEM: header, h_xll = b_xll + cellsize/2, cell
 * sizes (ComputeCellSize: projected metres, or degrees on a sphere of
 * radius 6378137 m, or the haversine extent for non-square cells). */
int rift_gridconfig_from_dem(const char* dem_path, int32_t square_cells, int32_t projected,
                             rift_gridconfig* gc);
/* GridConfig::Coord2Index; *ok = 0 when the index is outside the grid */
int rift_gridconfig_coord2index(const rift_gridconfig* gc, double X, double Y, int32_t* i,
                                int32_t* j, int32_t* ok);

/* ---- CSV time series (source.cc) --------------------------------------
 * '#' lines skipped; "hours, rate" -> seconds (float), rate (float); a zero
 * rate is appended at last + mean spacing when the last rate is not 0. */
int rift_csv_read(const char* path, float* times_s, float* rates, int32_t cap, int32_t* n);

/* ---- hot<k>.bin (simulator.cu:912-968, grid_config.cpp:124-170) --------
 * t, dt, GridConfig (98-byte header), w, hu, hv [, F] as FP64 h-grids,
 * wet_blocks[grow_grid_size] (bytes), active_blocks[grow_grid_size]
 * (int32, +id active / -id inactive, active first; tile 0 is 0). */
int64_t rift_hotstart_size(const rift_gridconfig* gc, int32_t has_F);
int rift_hotstart_write(const char* path, double t, double dt, const rift_gridconfig* gc,
                        const double* w, const double* hu, const double* hv, const double* F,
                        const uint8_t* wet_blocks, const int32_t* active_blocks);
/* reads into caller arrays of the sizes gc (read from the file) implies;
 * pass NULL pointers first to learn gc */
int rift_hotstart_read(const char* path, double* t, double* dt, rift_gridconfig* gc,
                       int32_t has_F, double* w, double* hu, double* hv, double* F,
                       uint8_t* wet_blocks, int32_t* active_blocks);
/* GrowGridSize of a grid (grid.cu:476-479) */
int32_t rift_grow_grid_size(int32_t h_nx, int32_t h_ny);

/* ---- the Simulator life cycle (simulator.cu) --------------------------- */
typedef struct rift_sim rift_sim;
/* OpenSimulation: ReadUserParams + InitSimulation (+ ReadHotstart).  On
 * failure *out is NULL and rift_host_last_error() holds the message. */
int rift_sim_open(const char* config_path, rift_sim** out);
/* RunSimulation: one step, map series updates, outputs when t > t_print */
int rift_sim_step(rift_sim* s, double* t);
/* RunSimulation repeated until t >= t_end (or tf), with the same outputs,
 * running the steps between two output / map events in one engine call */
int rift_sim_run(rift_sim* s, double t_end, double* t, int64_t* steps);
int rift_sim_time(rift_sim* s, double* t, double* dt, double* tf);
/* the engine handle, for direct field access */
rift_handle* rift_sim_engine(rift_sim* s);

/* ---- 1D-2D coupling hooks (simulator.h:133-137, simulator.cu:720-735,
 * 858-907) ------------------------------------------------------------------
 * OpenSimulation(config, flowrate): rift_sim_open, keeping the flow rate the
 * caller passes (the reference stores it in flow_rate and reads it nowhere
 * else; rift_sim_flow_rate returns it). */
int rift_sim_open_flow(const char* config_path, double flow_rate, rift_sim** out);
int rift_sim_flow_rate(rift_sim* s, double* flow_rate);
/* NumSources: cells of the point / rectangular source (InitializeSources) */
int rift_sim_num_sources(rift_sim* s, int32_t* n);
/* setSourceValue(value): a discharge in m^3/s spread over the source cells,
 * value / dx / dy / NumSources m/s each; with check_volume, each cell's rate
 * times the current dt is added to V_added (rift_sim_source_volume).  Takes
 * effect on the device at rift_sim_update_sources. */
int rift_sim_set_source_value(rift_sim* s, double value);
/* updateSources(): the rates to the device for the next step.  With a
 * hydrograph CSV in the configuration the next step's UpdateSource replaces
 * them from the hydrograph, as in the reference (simulator.cu:502-518); a
 * configuration that gives the source location (source_pt, source_X/Y or
 * source_rect_X/Y) without a hydrograph keeps them: the coupling's own
 * source. */
int rift_sim_update_sources(rift_sim* s);
/* V_added of setSourceValue (m of depth summed over cells x s; times dx dy
 * for m^3): the reference's check_volume bookkeeping of the set rates */
int rift_sim_source_volume(rift_sim* s, double* v_added);
/* CloseSimulation: summary maps, then frees everything */
int rift_sim_close(rift_sim* s);
const char* rift_sim_last_error(rift_sim* s);

#ifdef __cplusplus
}
#endif
#endif
