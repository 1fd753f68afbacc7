/* Internal layout shared by the SW2D device kernels and the host driver.
 *
 * Grid layout in HBM: every per-cell field is a row-major array of
 * (rows + 2*SW2D_HALO) rows of `pitch` elements; interior cell (r, c) sits at
 * (r + SW2D_HALO) * pitch + (c + SW2D_HALO).  The halo cells are inactive,
 * dry and carry zero discharge, which turns the reference's raster-edge
 * rules (walls on the edge and next to NODATA cells, SW2D-EFDC.cu:115, :231,
 * :657) into the single "both cells active" rule.  The pitch is a multiple of
 * 32 elements so every row starts on a 128-byte (FP32) / 256-byte (FP64)
 * boundary for coalesced and vectorised access.
 *
 * Face fields share the cell indexing: qx at index i is the x face NORTH of
 * cell i (the reference's um, positive southward), qy at index i the y face
 * WEST of cell i (the reference's vn, positive eastward).  The south edge of
 * the last row and the east edge of the last column live in the halo.
 */
#ifndef SW2D_INTERNAL_H
#define SW2D_INTERNAL_H

#include <stdint.h>
#include <cuda_runtime.h>

#define SW2D_HALO 2
#define SW2D_MAX_SRC 64
#define SW2D_BX 32
#define SW2D_BY 8

/* per-cell flag bits */
#define SW2D_F_ACTIVE 1u
#define SW2D_F_SOURCE 2u

namespace sw2d {

/* Forcing and length of one iteration, prepared on the device by the
 * previous iteration so that a captured sequence of iterations needs no host
 * round trip. */
struct Slot {
    double t;        /* start time */
    double t_mid;    /* time of the second forcing evaluation */
    double t_next;   /* start time of the following iteration */
    double dt2;      /* iteration length (the reference's dt2) */
    double dt2dx, dt2dy;
    double rr1, rr2; /* rain rate at t and t_mid, m/s */
    double ev1, ev2; /* evaporation rate at t and t_mid, m/s */
    int active;      /* 0: the loop condition failed, the iteration copies state */
    int pad;
    double ql1[SW2D_MAX_SRC], ql2[SW2D_MAX_SRC]; /* source rates, m/s */
};

enum {
    LED_VOLUME = 0, LED_VOLUME0, LED_RAIN, LED_SOURCE, LED_EVAP, LED_OUTFLOW, LED_CLAMP,
    LED_QOUT, LED_SMAX, LED_DTLAST, LED_N = 16
};

struct DevClock {
    Slot slot[2];
    double t;          /* current simulated time */
    double t_end;
    double s_max;      /* CFL speed of the current state */
    long long iters;
    double led[LED_N];
    unsigned int counter; /* last-block ticket of the reduction kernels */
    int status;           /* bit 0: non-finite volume seen */
    long long outlet_n;
    long long iter_end;   /* the slot after iteration iter_end is inactive (a state copy) */
};

/* Everything a step kernel needs, passed by value. */
struct StepParams {
    int R, C, P;
    int outflow_south;
    int dt_mode, series_mode;
    int nsrc, nrain, nevap, nq;
    int nblocks_cells;     /* blocks of the cell-grid reduction kernels */
    int outlet_cap;
    int ledger_cells;      /* 1: rain/evaporation volumes need a per-cell sum */
    double rain_static;    /* else: sum over active cells of weight * runoff fraction */
    double dx, dy, th, g, manning;
    double pct_lake, pct_land, ev_wl_min;
    double dtrain, dtoq, dt_fixed, cfl, dt_max, rdx, rdy, rsum, area;
    const uint8_t* flags;
    const double* z;
    const uint8_t* mcls;   /* Manning class per cell or NULL */
    const double* mtab;    /* class table (device) */
    const double* gnn;     /* (g n_f) n_f per (class, class) pair, ncls^2, or NULL */
    int ncls;
    double gnn_uni;        /* (g n) n of the uniform n */
    int kdx, kdy;          /* dx = 2^kdx (dy = 2^kdy) when a power of two >= 1, else -1 */
    const float* rainw;    /* rain weight per cell or NULL */
    const int* src_idx;    /* padded cell index per source */
    const double* rain;    /* nrain + 2 */
    const double* evap;    /* nevap + 2 or NULL */
    const double* srcq;    /* (nq + 2) * nsrc */
    double* h[2];
    double* qx[2];
    double* qy[2];
    double* uu1;
    double* vv1;
    double* partials;      /* nblocks_cells * 4: rain, evaporation, outlet sums */
    double* partials_f;    /* nblocks_faces * 2: CFL face-speed maxima (bit patterns) */
    int nblocks_faces;
    double* outlet;        /* outlet_cap * 2 or NULL */
    DevClock* clk;
};

/* FP64 step kernels (sw2d_fp64.cu) */
void fp64_launch_iteration(const StepParams& p, int cur, cudaStream_t s, cudaEvent_t* ev);
void fp64_launch_prime(const StepParams& p, int cur, int full, cudaStream_t s);
void fp64_launch_face_velocity(const StepParams& p, int cur, cudaStream_t s);
void fp64_launch_cell_velocity(const StepParams& p, int cur, double* uu, double* vv, double* uua,
                               double* vva, cudaStream_t s);
int fp64_kernels_per_iteration();

} // namespace sw2d

#endif
