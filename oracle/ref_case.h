/* Test infrastructure only: the case and result records shared by the
 * drivers of the reference's own kernels (ref_driver.cpp on the CPU,
 * ref_gpu_driver.cu on the GPU) and the ctypes mirror in oracle.py. */
#ifndef SW2D_REF_CASE_H
#define SW2D_REF_CASE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sw2dref_case {
    int rows, cols;
    double cellsize, nodata;
    const double* dem;     /* rows*cols, reference layout (row 0 = first ESRI line) */
    const double* h0;      /* rows*cols initial depth */
    double dt;             /* setup.dat TIME STEP; one iteration advances 2*dt */
    double time0, timmax;
    double manning;
    const double* rain;    /* rain.dat values, mm per dtrain */
    int nrain;
    double dtrain;
    double frac_int, frac_inf, frac_lwl, ev_wl_min;
    int evaporation_on;
    const double* temp;    /* nrain entries (temperatures.dat) */
    const double* rad;     /* nrain entries (solar_radiation.dat) */
    double albedo;
    int nst;               /* point sources */
    const double* brx;     /* nst, in cells (coordinate / cellsize) */
    const double* bry;
    const double* qq;      /* nqq*nst, Q_source_sink.dat rows, m3/s */
    int nqq;
    double dtoq;
    double xcoor_c, ycoor_c; /* xllcorner/cellsize, yllcorner/cellsize */
    const int* mask;       /* rows*cols coupling mask (1 = lake) or NULL */
    int lkout;             /* coupling interval in half-steps (mstep units) */
    double efdc_basetime;
    int max_samples;       /* rows of *_val the caller reserved */
    int nthreads;
    int warm_iters;        /* iterations excluded from loop_seconds */
} sw2dref_case;

typedef struct sw2dref_out {
    double *h, *um, *vn, *uu, *vv, *uua, *vva; /* N = rows*cols + cols/2 each, or NULL */
    long long iters;
    double time;
    int water_cells;
    int nqs;                 /* Qnqs after the last coupling sample */
    int nsamples;            /* tq + 1 */
    int* bc;                 /* 4 sides (N,S,E,W) x water_cells x 3, or NULL */
    double* val;             /* 4 sides x max_samples x (water_cells+1), or NULL */
    double loop_seconds;     /* wall time of the iterations after warm_iters */
} sw2dref_out;

#ifdef __cplusplus
}
#endif
#endif
