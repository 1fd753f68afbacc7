/* sw2d_batch.h -- batched and served FP32 SW2D through one C ABI.
 *
 * The reference advances one raster per process and has no batching or
 * request interface: main() loops over the cases listed in db/dir.txt one
 * after the other (SW2D-EFDC.cu:3733-3738) and calls the step kernels of
 * SW2D-EFDC.cu:97-725 for each.  This interface runs many scenarios of
 * uneven raster sizes together on one GPU: every iteration is one launch of
 * the FP32 row-marching kernel over all running scenarios of a feature class
 * (class raster, rain field, ...; one launch per class present) and one
 * finalize launch, each scenario with its own CFL iteration length and
 * forcing.
 *
 * Requests are admitted as HBM (the budget given at creation) and running
 * slots free up; their state stays on the device until they reach their end
 * time, when the final fields move to host memory and the device memory is
 * released.  One batch is driven by one host thread at a time.
 */
#ifndef SW2D_BATCH_H
#define SW2D_BATCH_H

#include <stdint.h>

#include "sw2d.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { SW2D_REQ_QUEUED = 0, SW2D_REQ_RUNNING = 1, SW2D_REQ_DONE = 2, SW2D_REQ_FAILED = 3 };

/* One scenario: the fields of sw2d_config plus its inputs.  Host arrays are
 * copied by sw2d_batch_submit. */
typedef struct sw2d_scenario {
    int rows, cols;
    int dt_mode;              /* SW2D_DT_* */
    int series_mode;          /* SW2D_SERIES_* */
    int outflow;              /* SW2D_OUTFLOW_* */
    int ntable;               /* Manning classes (<= 64), 0 = uniform */
    int nrain;
    int outlet_capacity;      /* outlet hydrograph ring, 0 = none */
    double dx, dy, nodata, th, g, manning;
    double dt, cfl, dt_max, t0, t_end;
    double frac_int, frac_inf, frac_lwl, ev_wl_min;
    double dtrain;
    const double* dem;        /* rows*cols, row 0 = north */
    const double* depth;      /* rows*cols or NULL (dry) */
    const uint8_t* manning_class;
    const double* manning_table;
    const double* rain_mm;    /* nrain values, mm per dtrain */
    const float* rain_weight; /* rows*cols or NULL */
} sw2d_scenario;

typedef struct sw2d_batch_stats {
    int running, queued;
    int work_items;           /* tiles per iteration */
    int rows_per_item;        /* rows of a work item in use (the autotuner's choice unless set) */
    double bytes_in_use;
    double device_ms;         /* device time of all iterations so far */
    double cell_updates;      /* sum over scenarios of cells x iterations advanced */
    double launches;          /* kernel launches issued (one persistent launch per feature class and chunk) */
    double tuning_ms;         /* host time the autotuner spent timing candidate work items (its timed
                                 iterations advanced the scenarios like any other) */
    int ctas_per_sm;          /* CTAs per SM of the persistent launches (the autotuner's choice; 0 = all
                                 that fit) */
    int tunings;              /* size buckets the autotuner has timed (each is cached) */
    double tuning_iterations; /* iterations sw2d_batch_tune advanced (in neither device_ms nor cell_updates) */
} sw2d_batch_stats;

typedef struct sw2d_batch sw2d_batch;

/* max_running = 0: no limit besides the HBM budget (0 = no budget). */
int sw2d_batch_create(int device, double hbm_budget_bytes, int max_running, sw2d_batch** out);
int sw2d_batch_destroy(sw2d_batch* b);
int sw2d_batch_submit(sw2d_batch* b, const sw2d_scenario* s, int64_t* id_out);
/* Admit what fits, advance every running scenario by `iterations`
 * iterations, retire the finished ones. */
int sw2d_batch_step(sw2d_batch* b, int iterations, int* n_running_out, int* n_queued_out);
/* Status of a request and its ledger: as of now for a running request
 * (read from the device: time, iterations, volumes so far), final for a
 * finished one, zeros for a queued one. */
int sw2d_batch_poll(sw2d_batch* b, int64_t id, int* status, sw2d_ledger* ledger);
/* Final fields of a finished request: depth rows*cols, qx (rows+1)*cols,
 * qy rows*(cols+1), reference orientation; any pointer may be NULL. */
int sw2d_batch_result(sw2d_batch* b, int64_t id, double* depth, double* qx, double* qy);
int sw2d_batch_release(sw2d_batch* b, int64_t id);
/* Rows per work item (a multiple of 4 in 16..512) for every scenario of the
 * batch; 0 (the default) lets the autotuner choose the work split: for a
 * work set of at least 1 M cells it times each pair of 64, 128, 256 or 512
 * rows per item and all or all-but-one CTAs per SM on the scenarios' own
 * iterations (one untimed, then up to 32 in one launch, within the
 * iterations of the sw2d_batch_step call that needs it) and keeps the
 * fastest, cached per size bucket (log2 of the running scenarios' cells).
 * Results do not depend on the choice (the bed's datum tiles are fixed at
 * 224 columns x 64 rows), so a scenario's results are the same alone and in
 * any mix. */
int sw2d_batch_set_rows_per_item(sw2d_batch* b, int rows);
/* Admit what fits and run the autotuner now for the running scenarios'
 * size bucket, advancing them by at most max_iterations iterations
 * (*iterations_out; 0 when the bucket is tuned already, rows per item are
 * fixed, the work set is under 1 M cells or max_iterations is below 24).
 * Finished scenarios are retired.  Lets a caller keep the tuning out of the
 * steps it times; those iterations count in neither device_ms nor
 * cell_updates of the stats. */
int sw2d_batch_tune(sw2d_batch* b, int max_iterations, int* iterations_out);
int sw2d_batch_get_stats(sw2d_batch* b, sw2d_batch_stats* out);
const char* sw2d_batch_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* SW2D_BATCH_H */
