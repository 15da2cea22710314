/*
 * rift_oracle.h -- CPU oracle for the RIFT shallow-water step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library; the
 * product path (rift_gb300) never links or calls it.
 *
 * A plain FP64 C++ restatement of the reference's device step (grid.cu) and
 * of the host pieces it depends on (simulator.cu ComputeTimestep,
 * RunSimulation order, source interpolation).  Two arithmetic modes:
 *   RIFT_ORACLE_REF    -- mirrors every float rounding point of the reference
 *                         (fminf/fmaxf/fabsf/sqrtf/powf on double arguments,
 *                         float literals, float source rates), with the host's
 *                         correctly rounded float functions standing in for
 *                         CUDA's fast-math ones;
 *   RIFT_ORACLE_PURE64 -- the same scheme with every rounding point in double.
 * Both keep the reference's low-word signf (grid.cu:62-71), so the limiter is
 * the reference's effective one, not a textbook minmod.
 *
 * The call surface mirrors include/rift_gb300.h (rift_oracle_* in place of
 * rift_*) so one test harness drives both.
 */
#ifndef RIFT_ORACLE_H
#define RIFT_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/rift_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RIFT_ORACLE_REF    0
#define RIFT_ORACLE_PURE64 1

typedef struct rift_oracle rift_oracle;

int rift_oracle_create(const rift_grid_desc* g, int32_t mode, rift_oracle** out);
int rift_oracle_upload_static(rift_oracle* o, const double* BX, const double* BY,
                              const double* n, const double* K_mps, const double* h0);
int rift_oracle_init(rift_oracle* o, double t0);
int rift_oracle_set_uniform_rates(rift_oracle* o, double rain_mps, double drain_mps);
int rift_oracle_set_point_sources(rift_oracle* o, const int32_t* idx,
                                  const double* rate_mps, int32_t n);
int rift_oracle_set_map(rift_oracle* o, int32_t which, const double* t0map,
                        const double* t1map, double factor);
int rift_oracle_set_map_factor(rift_oracle* o, int32_t which, double factor);
int rift_oracle_set_map_times(rift_oracle* o, int32_t which, double t0, double t1);
int rift_oracle_set_series(rift_oracle* o, int32_t which, const float* times_s,
                           const float* rates, int32_t n);
int rift_oracle_step(rift_oracle* o, double* t, double* dt);
int rift_oracle_run(rift_oracle* o, int32_t nsteps, double t_stop, double* t,
                    double* dt, int32_t* steps_done);
int rift_oracle_get_field(rift_oracle* o, int32_t which, double* host, size_t ld);
int rift_oracle_get_tiles(rift_oracle* o, uint8_t* wet, int32_t* active, int32_t* n_active);
int rift_oracle_get_tile_speeds(rift_oracle* o, double* mx, double* my);
int rift_oracle_set_state(rift_oracle* o, double t, double dt_prev, const double* w,
                          const double* hu, const double* hv, const double* F,
                          const uint8_t* wet, const int32_t* active_ids, int32_t n_active,
                          const double* mx, const double* my);
int rift_oracle_get_time(rift_oracle* o, double* t, double* dt);
int rift_oracle_volume(rift_oracle* o, double* volume);
int rift_oracle_mass_ledger(rift_oracle* o, double* volume, double* added);
/* The full FP64 ledger (rift_ledger of include/rift_gb300.h), since
 * rift_oracle_init / rift_oracle_set_state; always kept. */
int rift_oracle_mass_ledger_terms(rift_oracle* o, rift_ledger* out);
int rift_oracle_get_tile_grid(rift_oracle* o, int32_t* nBX, int32_t* nBY);
int rift_oracle_set_threads(int32_t n);
const char* rift_oracle_last_error(rift_oracle* o);
void rift_oracle_destroy(rift_oracle* o);

/* Pure device-math probes (no grid): used to pin the limiter semantics. */
double rift_oracle_minmod(double a, double b, double c);
double rift_oracle_limiter(double U, double Up1, double Um1);

#ifdef __cplusplus
}
#endif
#endif
