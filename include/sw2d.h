/* sw2d.h -- C ABI of the GB300-native SW2D explicit 2-D overland step.
 *
 * The reference (LabHidro/SW2D-EFDC, SW2D-EFDC.cu) has no library API: its
 * hot path is a set of CUDA kernels taking raw device arrays of length
 * N = rows*cols + cols/2 plus scalars (SW2D-EFDC.cu:97-100, :602, :695),
 * driven by main() (time loop SW2D-EFDC.cu:4798-4878).  This header is the
 * drop-in boundary for that path: plain pointers and sizes, host buffers in
 * the reference's orientation (row-major, row 0 = first line of the ESRI
 * grid, i.e. north), every call returning an int status.
 *
 * Threading: one handle is driven by one host thread at a time; different
 * handles may be driven concurrently.  A handle owns its device memory.
 * Caller-owned host buffers are only read or written during a call.
 */
#ifndef SW2D_H
#define SW2D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SW2D_ABI_VERSION 2

/* Status codes.  The reference checks no error at all (no cudaGetLastError,
 * missing files print and return 0, SW2D-EFDC.cu:3757-3761). */
enum {
    SW2D_OK = 0,
    SW2D_ERR_INVALID = -1,   /* bad argument or configuration */
    SW2D_ERR_CUDA = -2,      /* CUDA runtime error (message in sw2d_last_error) */
    SW2D_ERR_NOMEM = -3,     /* device or host allocation failed */
    SW2D_ERR_STATE = -4,     /* call not valid in the handle's current state */
    SW2D_ERR_BUDGET = -5,    /* request exceeds the configured HBM budget */
    SW2D_ERR_NUMERIC = -6,   /* non-finite depth or discharge detected */
    SW2D_ERR_NODEVICE = -7,  /* no CUDA device of compute capability 10.3 */
    SW2D_ERR_TIMEOUT = -8,   /* a bounded device wait gave up */
    SW2D_ERR_NOT_FOUND = -9, /* unknown request id */
    SW2D_ERR_IO = -10        /* a file could not be opened or written */
};

/* Arithmetic of the state and fluxes. */
enum { SW2D_FP64 = 0, SW2D_FP32 = 1 };

/* Iteration length.  FIXED is the reference's: dt from setup.dat, one
 * iteration advances 2*dt (SW2D-EFDC.cu:3976, :4838, :4876).  CFL sets each
 * iteration's length to min(dt_max, cfl / s) with
 * s = max over wet cells of (|qx_c|/dx + |qy_c|/dy)/h + sqrt(g h)(1/dx + 1/dy). */
enum { SW2D_DT_FIXED = 0, SW2D_DT_CFL = 1 };

/* Interpolation of the rain, evaporation and point-source series.
 * REFERENCE reproduces SW2D-EFDC.cu:546-553 exactly (ramp for t <= 1 s and
 * the interpolation that divides by the elapsed time); LINEAR interpolates
 * linearly between entries; STEP holds each entry over its interval. */
enum { SW2D_SERIES_REFERENCE = 0, SW2D_SERIES_LINEAR = 1, SW2D_SERIES_STEP = 2 };

/* Open boundaries.  The reference has walls on every raster edge
 * (SW2D-EFDC.cu:115, :231); SOUTH opens the last row's south faces as a free
 * overfall q = 0.544 h sqrt(g h) (the reference's own dry-bed weir law). */
enum { SW2D_OUTFLOW_NONE = 0, SW2D_OUTFLOW_SOUTH = 1 };

typedef struct sw2d_config {
    int rows, cols;          /* raster size (ESRI nrows, ncols) */
    int precision;           /* SW2D_FP64 or SW2D_FP32 */
    int dt_mode;             /* SW2D_DT_* */
    int series_mode;         /* SW2D_SERIES_* */
    int outflow;             /* SW2D_OUTFLOW_* */
    int device;              /* CUDA device ordinal */
    int reserved0;
    double dx, dy;           /* cell size; the reference uses dx = dy = cellsize */
    double nodata;           /* ESRI NODATA_value; such DEM cells are inactive */
    double th;               /* wet/dry threshold, 1e-4 m (SW2D-EFDC.cu:4644) */
    double g;                /* 9.80 (SW2D-EFDC.cu:3977) */
    double manning;          /* uniform Manning n (setup.dat MANNING COEFFICIENT) */
    double dt;               /* SW2D_DT_FIXED: setup.dat TIME STEP (iteration = 2 dt) */
    double cfl;              /* SW2D_DT_CFL: Courant number */
    double dt_max;           /* SW2D_DT_CFL: cap on the iteration length */
    double t0;               /* start time, s */
    double frac_int;         /* setup.dat interception fraction (INT) */
    double frac_inf;         /* setup.dat infiltration fraction (INF) */
    double frac_lwl;         /* setup.dat lake water-loss fraction (LWL) */
    double ev_wl_min;        /* setup.dat minimum depth for evaporation */
    double hbm_budget_bytes; /* 0 = no limit */
} sw2d_config;

typedef struct sw2d_ledger {
    double time;             /* simulated time, s */
    double iterations;       /* iterations advanced */
    double volume;           /* sum of h dx dy over active cells, m3 */
    double volume0;          /* volume at the last set_depth/restore */
    double rain_in;          /* cumulative rain volume, m3 */
    double source_in;        /* cumulative point-source volume, m3 */
    double evap_out;         /* cumulative evaporation volume, m3 */
    double outflow;          /* cumulative outlet volume, m3 */
    double clamp_gain;       /* volume created by the max(h,0) clamp, m3 */
    double q_out;            /* outlet discharge of the last iteration, m3/s */
    double s_max;            /* last CFL speed maximum, 1/s */
    double dt_last;          /* length of the last iteration, s */
    double balance_error;    /* (volume - volume0 - rain_in - source_in + evap_out
                                + outflow) / max(rain_in + source_in, tiny) */
} sw2d_ledger;

typedef struct sw2d_handle sw2d_handle;

/* Defaults: th 1e-4, g 9.80, manning 0.03, FP64, FIXED dt 0.04, REFERENCE
 * series, no outflow, device 0, nodata -9999. */
int sw2d_config_default(sw2d_config* cfg);

/* Allocate a model on the configured device.  Replaces the reference's
 * cudaMalloc block SW2D-EFDC.cu:4677-4704 and init_inf/initiald :29-91. */
int sw2d_create(const sw2d_config* cfg, sw2d_handle** out);
int sw2d_destroy(sw2d_handle* h);

/* Bed elevation, rows*cols doubles (dem.dat, SW2D-EFDC.cu:3983-4003);
 * cells equal to cfg.nodata are inactive (init_inf, SW2D-EFDC.cu:37-42). */
int sw2d_set_dem(sw2d_handle* h, const double* z);
/* Initial depth, rows*cols doubles (initial_condition.dat, SW2D-EFDC.cu:4170-4181).
 * Resets discharges to zero, the clock to cfg.t0 and the volume ledger. */
int sw2d_set_depth(sw2d_handle* h, const double* depth);
/* Per-cell Manning n as a class raster and a table (face n = mean of the two
 * cells).  The reference has one scalar n (rn, SW2D-EFDC.cu:4810).  NULL
 * classes restores the uniform cfg.manning. */
int sw2d_set_manning_classes(sw2d_handle* h, const uint8_t* classes, const double* table, int ntable);
/* Per-cell Manning n as rows*cols values; NULL restores the uniform
 * cfg.manning.  Stored as the class raster of its distinct values
 * (sw2d_manning_classes_of), which gives the same face coefficients: at most
 * 256 distinct values on FP64 handles, 64 on FP32 handles. */
int sw2d_set_manning_field(sw2d_handle* h, const double* n);
/* Rain series: n values in mm per dtrain seconds (rain.dat, SW2D-EFDC.cu:4078-4108). */
int sw2d_set_rain_series(sw2d_handle* h, const double* mm, int n, double dtrain);
/* Per-cell rain weight (rows*cols floats) multiplying the series rate; NULL = 1. */
int sw2d_set_rain_field(sw2d_handle* h, const float* weight);
/* Evaporation series in mm per dtrain (the Evapo series of
 * gpu_evaporation_calc, SW2D-EFDC.cu:556-586), applied where ho > ev_wl_min. */
int sw2d_set_evaporation_series(sw2d_handle* h, const double* mm, int n);
/* Point sources/sinks: nsrc raster cell ids (row*cols + col) and nq rows of
 * nsrc discharges in m3/s every dtoq seconds (Q_source_sink.dat,
 * SW2D-EFDC.cu:4008-4070 and stream_flow :531-545).  At most 64 sources. */
int sw2d_set_point_sources(sw2d_handle* h, int nsrc, const int* cells, const double* q, int nq,
                           double dtoq);

/* Advance until the loop condition fails: FIXED runs the reference's
 * while (time + dt <= t_end) loop, CFL advances until time == t_end (the last
 * iteration is shortened).  iterations_out may be NULL. */
int sw2d_advance(sw2d_handle* h, double t_end, int64_t* iterations_out);
/* Advance exactly n iterations (or fewer if t_end is reached). */
int sw2d_step(sw2d_handle* h, int n, double t_end);
int sw2d_get_time(sw2d_handle* h, double* t, int64_t* iterations);

/* State in the reference orientation.  depth: rows*cols.  qx: (rows+1)*cols
 * x-face discharges (row r = face north of cell row r, the reference's um;
 * row rows = south edge).  qy: rows*(cols+1) y-face discharges (the
 * reference's vn; column cols = east edge).  Any pointer may be NULL. */
int sw2d_get_state(sw2d_handle* h, double* depth, double* qx, double* qy);
/* Cell velocities as the reference's uu_vv kernel (SW2D-EFDC.cu:458-483):
 * uu along rows (VTK y_velocity = -uu), vv along columns (VTK x_velocity = vv). */
int sw2d_get_velocity(sw2d_handle* h, double* uu, double* vv);
/* Cross-face velocities uua (at y faces) and vva (at x faces), rows*cols each,
 * as uua_vva (SW2D-EFDC.cu:489-522). */
int sw2d_get_face_velocity(sw2d_handle* h, double* uua, double* vva);
int sw2d_get_ledger(sw2d_handle* h, sw2d_ledger* out);
/* Outlet hydrograph recorded on the device, one (t, Q) pair per iteration in
 * a ring of `capacity` entries (set with sw2d_set_outlet_record).  count_out
 * receives the number of pairs written (at most capacity, oldest first). */
int sw2d_set_outlet_record(sw2d_handle* h, int capacity);
int sw2d_get_outlet(sw2d_handle* h, double* t, double* q, int capacity, int* count_out);

/* Boundary-discharge hand-off to EFDC (couple_BC_efdc, SW2D-EFDC.cu:728-1067).
 * set_coupling_mask: rows*cols ints, 1 = lake.  Builds the boundary-face list
 * in the reference's scan order; n_faces_out receives its length.
 * lagged = 1 reproduces the reference's use of the previous sample's
 * velocities (SW2D-EFDC.cu:4909-4916); 0 uses the current ones. */
int sw2d_set_coupling_mask(sw2d_handle* h, const int* mask, int lagged, int* n_faces_out);
/* Face list: side (0 north, 1 south, 2 east, 3 west as the reference's
 * north_bc..west_bc arrays), EFDC I and J (1-based), raster cell id. */
int sw2d_get_coupling_faces(sw2d_handle* h, int* side, int* efdc_i, int* efdc_j, int* cell, int capacity);
/* The same face list for a lake mask (rows*cols, 1 = lake) without a handle:
 * *n_out faces, the first `capacity` of them written (any output may be
 * NULL).  Host only. */
int sw2d_coupling_faces_of(int rows, int cols, const int* mask, int* side, int* efdc_i, int* efdc_j, int* cell,
                           int capacity, int* n_out);
/* Take one coupling sample at the current state; when initial is nonzero the
 * depths are the initial condition and the velocities zero, as the
 * reference's first sample (SW2D-EFDC.cu:4905).  q_out: n_faces discharges
 * (m3/s, inflow to the lake only), may be NULL. */
int sw2d_couple_sample(sw2d_handle* h, int initial, double* q_out, int capacity);
/* Write the EFDC inflow deck QSER.INP as write_efdc_QSER does
 * (SW2D-EFDC.cu:2499-2610, read by EFDC_src/INPUT.F:3969-4010), byte for byte:
 * one series per coupling face, north faces first, then south, east, west.
 * side: n_faces sides from sw2d_get_coupling_faces; times: nsamples values of
 * the first column (the reference's mstep*dt / efdc_basetime); q: nsamples
 * rows of n_faces discharges from sw2d_couple_sample; each of the nlayers
 * layers receives q / nlayers; type is the deck's InType. Host only. */
int sw2d_write_qser(const char* path, int type, int nlayers, double efdc_basetime, int n_faces, const int* side,
                    int nsamples, const double* times, const double* q);
/* The dye, temperature and salinity decks of the same inflows, DSER.INP,
 * TSER.INP, SSER.INP (kind 'D', 'T', 'S'), as write_efdc_DSER / _TSER / _SSER
 * write them (SW2D-EFDC.cu:2383-2498, :2141-2254, :2026-2140), byte for byte:
 * every layer of sample t of every face carries value[t] (nsamples values;
 * the reference passes one concentration for dye and salt, a series for
 * temperature). Host only. */
int sw2d_write_efdc_concentration(const char* path, char kind, int type, int nlayers, double efdc_basetime,
                                  int n_faces, const int* side, int nsamples, const double* times,
                                  const double* value);
/* Rewrite, in place in an existing EFDC.INP, the cards that depend on the
 * boundary-face list, as write_efdc_CONFIG does (SW2D-EFDC.cu:1476-1766):
 * C22 (number of salinity / temperature / dye series), C23 (NQSIJ, NQSER),
 * C24 (one source row per face: north faces first, then south, east, west),
 * C25 and C26 (one row of zeros per face).  Each card is replaced with the
 * reference's own file surgery (find the card's first token and the next
 * card's, write the new card, move the rest of the file behind it, blank
 * the shortfall), so the file is byte for byte the one the reference
 * leaves.  Faces as sw2d_get_coupling_faces returns them; salt_on, temp_on,
 * dye_on are the setup.dat switches.  Host only. */
int sw2d_write_efdc_cards(const char* path, int n_faces, const int* side, const int* efdc_i, const int* efdc_j,
                          int salt_on, int temp_on, int dye_on);
/* The DEM pre-pass of a coupled run (lake_catchment_smooth,
 * SW2D-EFDC.cu:2766-2827), in place on rows*cols elevations in the
 * reference orientation: catchment cells next to the lake mask (1 = lake)
 * take the mean of their two neighbours across the mask edge, in the
 * reference's sweep order (last raster row first, each row west to east,
 * updated values feeding later cells).  Host only. */
int sw2d_lake_catchment_smooth(int rows, int cols, const int* mask, double* dem);
/* The same DEM pre-pass on the device, in place on caller-owned device
 * arrays (d_mask: rows*cols ints, d_dem: rows*cols doubles, reference
 * orientation), on `stream` (NULL = the legacy default stream): the lake-edge
 * cells listed per anti-diagonal, then a wavefront over the diagonals, which
 * keeps the reference's sweep order (a cell reads its south and west
 * neighbours after their update), bit-identical to sw2d_lake_catchment_smooth.
 * Allocates a scratch list of the edge cells; synchronizes `stream` before
 * it returns.  Replaces the host loop of SW2D-EFDC.cu:2766-2827. */
int sw2d_lake_catchment_smooth_device(int rows, int cols, const int* d_mask, double* d_dem, void* stream);
/* Evaporation series for sw2d_set_evaporation_series: n values in mm per
 * dtrain from air temperature (deg C) and global radiation (W/m2), by the
 * energy-balance method of gpu_evaporation_calc (SW2D-EFDC.cu:556-586),
 * negative values clipped to zero.  Host only. */
int sw2d_evaporation_series(int n, const double* temp, const double* rad, double albedo, double dtrain,
                            double* mm_out);

/* A per-cell Manning field as classes: table = its distinct values in
 * ascending order (*ntable_out of them, at most max_classes <= 256),
 * classes[k] = the index of field[k] in table.  Values must be finite and
 * >= 0.  SW2D_ERR_INVALID when the field has more than max_classes distinct
 * values.  Host only. */
int sw2d_manning_classes_of(int64_t count, const double* field, int max_classes, uint8_t* classes, double* table,
                            int* ntable_out);

/* Device state snapshot (h, qx, qy, clock, ledger) to a host buffer. */
int sw2d_snapshot_size(sw2d_handle* h, size_t* bytes);
int sw2d_snapshot(sw2d_handle* h, void* buf, size_t bytes);
int sw2d_restore(sw2d_handle* h, const void* buf, size_t bytes);

/* Mean device time per iteration (ms) of the kernels launched by the last
 * sw2d_advance/sw2d_step, measured with CUDA events on the handle's stream;
 * kernel_ms_out (may be NULL) receives per-kernel means in launch order and
 * nkernels_out their count. */
int sw2d_get_timing(sw2d_handle* h, double* ms_per_iteration, double* kernel_ms_out, int* nkernels_out);
/* Enable per-kernel event timing for subsequent advances (slower; 0 = off). */
int sw2d_set_profiling(sw2d_handle* h, int on);

/* Thread-local message of the last failing call. */
const char* sw2d_last_error(void);
const char* sw2d_status_string(int status);
int sw2d_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* SW2D_H */
