/* CPU restatement of HAIL-CAESAR's per-timestep raster path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * product (hail-caesar_gb300/csrc) and the CPU baseline of bench.py.  Nothing
 * in the product links, loads or calls it.
 *
 * Parity pinned: oracle/ref_harness.cpp runs the unmodified reference sources
 * on the same inputs; tests/test_oracle_pin.py and the committed fixtures in
 * tests/golden/ compare the two.  The Boscastle 50 m known-good answers of the
 * reference's own test suite (test/basic_kga_tests.py) are checked as well.
 *
 * State uses the reference's layouts (LSDCatchmentModel.cpp:1617-1843):
 *   padded 2-D fields  (imax+2) x (jmax+2) row-major, [i][j] = row i, col j
 *   vel_dir            (imax+2) x (jmax+2) x 9
 *   sr, sl, su, sd     (imax+2) x (jmax+2) x 10
 *   grain              (imax+2)(jmax+2) x 11   rows addressed by index[i][j]
 *   strata             (imax+2)(jmax+2) x 10 x 11
 *   down_scan          (jmax+2) x (imax+2)     [column j][k] = k-th wet row
 *   edge, edge2        (imax+1) x (jmax+1)
 *   veg                (imax+1) x (jmax+1) x 4
 */
#ifndef HC_ORACLE_H
#define HC_ORACLE_H

#include <stdint.h>
#include "../include/hc_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hco_model hco_model;

/* Per-iteration record, written by hco_iterate (same fields as the harness). */
typedef struct hco_step_record {
  double counter, cycle, time_step, maxdepth, waterOut, waterinput,
      erode_mult, sediQ, globalsediq, baseflow;
  double vol_in, vol_out, vol_mask, volume;  /* the water ledger, as in hc_step_record */
} hco_step_record;

hco_model* hco_create(const hc_params* p);
void hco_destroy(hco_model* m);

/* Field access by name ("elev", "water_depth", "qx", ... see hco_field). */
int64_t hco_field_size(hco_model* m, const char* name);  /* elements, -1 if unknown */
int hco_field_elsize(hco_model* m, const char* name);    /* bytes per element */
void* hco_field(hco_model* m, const char* name);          /* raw pointer */
double hco_get_scalar(hco_model* m, const char* name);
int hco_set_scalar(hco_model* m, const char* name, double v);

/* Time-series inputs.  rain: rows x cols floats (rain file, mm/h);
 * reach: point p, rows x cols floats (reach file). */
void hco_set_rain(hco_model* m, const float* rain, int rows, int cols);
void hco_set_reach(hco_model* m, int point, const float* data, int rows, int cols);

/* Mirrors load_data's post-processing (count_catchment_gridcells) and the
 * set-up sequence of main.cpp:102-122 (set_time_counters,
 * initialise_rainfall_runoff, initialise_drainage_area).  Call after the
 * fields are filled. */
void hco_prepare(hco_model* m);

/* Runs n iterations of the main.cpp:139-204 loop (stops early when
 * cycle/60 >= maxcycle).  flags: HC_RUN_LATERAL, HC_RUN_NOHILL.
 * Returns the number of iterations run. */
long hco_iterate(hco_model* m, long n, int flags, hco_step_record* rec);

/* Continue from a state loaded field by field (after the scalars are set). */
void hco_resume(hco_model* m);

/* Single members, for unit tests. */
void hco_flow_route(hco_model* m);
void hco_depth_update(hco_model* m);
void hco_scan_area(hco_model* m);
void hco_water_flux_out(hco_model* m);
double hco_erode(hco_model* m, double mult);
void hco_lateral_channel_erode(hco_model* m);
void hco_in_channel_landsliding(hco_model* m);
void hco_creep(hco_model* m, double time);
void hco_global_landsliding(hco_model* m);
void hco_set_maximum_timestep(hco_model* m);
double hco_get_flow_timestep(hco_model* m);

#ifdef __cplusplus
}
#endif
#endif
