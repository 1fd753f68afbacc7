/* Test infrastructure only: the CPU oracle of the SW2D explicit step.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it, as the checker; the shipped library never links or calls it.
 */
#ifndef SW2D_ORACLE_H
#define SW2D_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_MATH_LIBM = 0, ORC_MATH_DEVICE = 1 };
enum { ORC_DT_FIXED = 0, ORC_DT_CFL = 1 };
enum { ORC_RAIN_REFERENCE = 0, ORC_RAIN_LINEAR = 1, ORC_RAIN_STEP = 2 };

typedef struct orc_config {
    int rows, cols;
    int math;           /* ORC_MATH_* */
    int dt_mode;        /* ORC_DT_* */
    int rain_mode;      /* ORC_RAIN_* */
    int outflow_south;  /* free-overfall outlet on the last row's south faces */
    int nrain;
    int nsrc, nq;
    int nevap;
    int nthreads;
    double dx, dy, nodata;
    double th, g, manning;
    double dt;          /* fixed mode: the reference's dt; one iteration advances 2*dt */
    double cfl, dt_max; /* CFL mode: iteration length min(dt_max, cfl / s_max) */
    double t0;
    double dtrain;
    double frac_int, frac_inf, frac_lwl, ev_wl_min;
    double dtoq;
} orc_config;

typedef struct orc_ledger {
    double volume;      /* sum of h dx dy over active cells */
    double volume0;
    double rain_in;     /* cumulative rain volume applied by the final continuity */
    double source_in;   /* cumulative point-source volume */
    double evap_out;    /* cumulative evaporation volume */
    double outflow;     /* cumulative outlet volume */
    double clamp_gain;  /* volume created by the max(h, 0) clamp */
    double q_out;       /* outlet discharge of the last iteration, m3/s */
    double s_max;       /* last CFL speed sum max over wet cells (1/s) */
    double dt2_last;    /* last iteration length */
} orc_ledger;

typedef struct orc_state orc_state;

/* dem, h0: rows*cols, row 0 = first (north) ESRI row.
 * manning: rows*cols per-cell n or NULL (uniform cfg->manning).
 * rain_w: rows*cols per-cell rain weight or NULL (1).
 * rain: nrain values in mm per dtrain; evap: nevap values in mm per dtrain or NULL.
 * src_cell: nsrc raster cell ids; src_q: nq*nsrc discharges (m3/s), row-major in time. */
orc_state* orc_create(const orc_config* cfg, const double* dem, const double* h0,
                      const double* manning, const float* rain_w, const double* rain,
                      const double* evap, const int* src_cell, const double* src_q);
void orc_destroy(orc_state* s);

/* Advance one iteration; returns 1, or 0 when the fixed-dt loop condition
 * (time + dt <= t_end) or the CFL condition (time < t_end) fails. */
int orc_step(orc_state* s, double t_end);
/* Advance until the loop condition fails or max_iters iterations ran. */
long long orc_run(orc_state* s, double t_end, long long max_iters);

double orc_time(const orc_state* s);
long long orc_iters(const orc_state* s);
void orc_ledger_get(const orc_state* s, orc_ledger* out);

/* Fields in the reference orientation.
 * depth, uu, vv: rows*cols.  qx: (rows+1)*cols (row r = face north of cell row r;
 * row rows = the south edge).  qy: rows*(cols+1).  uua: rows*cols (y faces),
 * vva: rows*cols (x faces) as the reference's uua_vva kernel defines them. */
void orc_get_fields(const orc_state* s, double* depth, double* qx, double* qy, double* uu,
                    double* vv, double* uua, double* vva);

/* Outlet hydrograph: one (t_end_of_iteration, Q) pair per iteration so far. */
long long orc_outlet_count(const orc_state* s);
void orc_outlet_get(const orc_state* s, double* t, double* q);

/* Boundary-discharge hand-off (SW2D-EFDC.cu:728-1067) on a lake mask
 * (1 = lake).  Face list in the reference's scan order. */
int orc_couple_faces(int rows, int cols, const int* mask, int max_faces, int* side, int* ci,
                     int* cj, int* cell);
/* Discharge per face from depth h and velocity fields uua/vva (reference layout, rows*cols). */
void orc_couple_values(int rows, int cols, double dx, double dy, int nfaces, const int* side,
                       const int* cell, const double* h, const double* uua, const double* vva,
                       double* q);

#ifdef __cplusplus
}
#endif
#endif
