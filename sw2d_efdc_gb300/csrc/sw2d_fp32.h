/* FP32 precision form of the SW2D step: device-side structures shared by the
 * row-marching kernel (sw2d_fp32.cu) and the scenario engine (sw2d_engine.cu).
 *
 * One kernel serves the single-raster, batched and served forms: its work
 * list holds (scenario, column strip, row segment) items and every scenario
 * has its own descriptor, clock, iteration length and forcing.  The kernel
 * is persistent: one launch advances every scenario of its feature class by
 * a chunk of iterations, its CTAs taking items from a device queue in
 * iteration order; a scenario's items of iteration n+1 start once all of its
 * items of iteration n are done and the last of them has reduced the
 * scenario's partials (dataflow per scenario, no grid-wide barrier).
 *
 * Layout of a scenario in HBM: binary32 fields with a 4-cell halo
 * ((rows + 8) rows of `pitch` floats, pitch >= cols + 12 and a multiple of
 * 32), cell (r, c) at (r + 4) * pitch + (c + 4).  The bed is stored as
 * binary32 offsets from the datum of the cell's datum tile (224 columns x 64
 * rows, fixed whatever the work items' shape), a multiple of 1/16 m so that
 * datum differences are exact in binary32; a face's bed step is the
 * difference of its two offsets plus the difference of their datums (zero
 * inside a datum tile), so results do not depend on the work items' shape.
 * Inactive cells (NODATA and the halo) hold NaN as bed offset.  Manning
 * classes, when present, are one byte per cell.
 */
#ifndef SW2D_FP32_H
#define SW2D_FP32_H

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace sw2d {

constexpr int M_H = 4;                 /* halo */
constexpr int M_DR = 64;               /* rows of a datum tile (its columns: one strip, M_CW) */
constexpr int M_MAXSEG = 512;          /* longest work item (rows) */
constexpr int M_MAXBANDS = (M_MAXSEG + 6 + M_DR - 1) / M_DR + 1; /* datum bands one work item spans */
constexpr int M_NW = 4;                /* warps per CTA */
constexpr int M_SW = 56;               /* output columns per warp (2 per lane, lanes 2..29) */
constexpr int M_CW = M_NW * M_SW;      /* 224 output columns per strip */
constexpr int M_BW = M_CW + 2 * M_H;   /* 232 staged columns */
constexpr int M_RB = 4;                /* rows per staged block (TMA box height) */
constexpr int M_NS = 2;                /* blocks in the staging ring */
constexpr int M_NT = M_NW * 32;
constexpr int M_CLSW = 240;            /* staged Manning-class columns (bytes; a multiple of 16) */
constexpr int M_CLSR = M_RB + 2;       /* class rows per block: the block's rows and the two above */
constexpr int M_RWR = M_RB + 1;        /* rain-weight rows per block: from three rows above the block */
constexpr int T32_MAXCLASS = 64;
constexpr int T32_MAXSRC = 64;         /* point sources per scenario */

/* Length and forcing of a scenario's next iteration, written by the
 * finalize kernel, read by every work item of the scenario. */
struct Slot32 {
    float dt2, dt2dx, dt2dy;
    float rr1, rr2;     /* rain rate, m/s */
    float ev1, ev2;     /* evaporation rate, m/s */
    int active;
    int cur;            /* which of the two state buffers is current */
    int pad[7];
};

struct Clock32 {
    Slot32 slot;
    double t, t_end, dt2;     /* dt2: length of the iteration in flight */
    double s_max;
    long long iters;
    double rain_in, source_in, evap_out, outflow, clamp_gain, q_out;
    double volume0;
    int status;               /* bit 0 non-finite, bit 1 TMA wait timeout, bit 2 misaligned staging */
    int done;                 /* set when t reached t_end */
    long long outlet_n;
    float ql1[T32_MAXSRC], ql2[T32_MAXSRC]; /* point-source rates (m/s) at the slot's two times */
};

/* per work item reduction results */
struct Part32 {
    double rain;   /* sum of weight * runoff fraction over active cells (if per cell) */
    double clamp;  /* depth created by the max(h, 0) clamp */
    double qout;   /* outlet discharge per unit width summed over the edge faces */
    double evap;   /* active cells with ho > ev_wl_min (count) */
    float sx, sy;  /* CFL face-speed maxima of the entering state (x and y faces) */
    int pad[6];
};

struct Scn32 {
    CUtensorMap tm_h[2], tm_qx[2], tm_qy[2], tm_z, tm_kc;
    CUtensorMap tm_cls, tm_rw;   /* set when the scenario has a class raster / a rain-weight field */
    float* h[2];
    float* qx[2];
    float* qy[2];
    float* kc;             /* Kahan compensation of the depth */
    const float* z;        /* bed offset (NaN = inactive), the TMA-mapped array */
    const float* datum;    /* per datum tile, bands * tiles_x */
    const uint8_t* cls;    /* Manning class per cell (padded) or NULL */
    const float* rainw;    /* per cell (padded) or NULL */
    const double* rain;    /* nrain + 2, mm per dtrain */
    const double* evap;    /* nevap + 2 or NULL */
    const double* srcq;    /* point-source discharges, (nq + 2) rows of nsrc, m3/s, or NULL */
    const int* src_cell;   /* nsrc raster ids (row * C + col), distinct */
    double* outlet;        /* outlet ring (t, Q) or NULL */
    Clock32* clk;
    int R, C, P, tiles_x, tiles_y, seg, bands;
    int first_work, nwork;
    int outflow_south, ledger_cells, series_mode, dt_mode;
    int nrain, nevap, outlet_cap;
    int nsrc, nq;
    int stall_staging;     /* failure test: issue no staged loads, so the bounded wait runs out */
    double dtoq;
    float dx, dy, rdx, rdy, th, g;
    float pct_lake, pct_land, ev_wl_min;
    double rain_static;    /* sum over active cells of weight * runoff fraction */
    double dxd, dyd, dtrain, dt_fixed, cfl, dt_max, area;
    float ntab[T32_MAXCLASS];
};

/* Control block of one persistent launch (zeroed before it): the queue
 * ticket, the abort flag a CTA sets when a bounded wait runs out, and per
 * scenario the iterations completed in this launch and the items finished
 * of the current one. */
struct Ctl32 {
    unsigned int next;
    unsigned int abort;
    int pad[2];
};
inline size_t fp32_ctl_bytes(int nscn) { return sizeof(Ctl32) + 2 * sizeof(int) * (size_t)(nscn > 0 ? nscn : 1); }

/* Feature class of a scenario (bit 0 class raster, bit 1 rain-weight field,
 * bit 2 lake fraction or evaporation, bit 3 point sources): the marching
 * kernel is specialised per class and the work list holds each class's
 * items contiguously. */
constexpr int T32_NCLASS = 16;
int fp32_feature_class(const Scn32& d);
/* niter iterations of every scenario: per feature class present, one
 * persistent launch of `grid[k]` CTAs over its work items; d_ctl holds
 * fp32_ctl_bytes(nscn) bytes and is cleared first.  Returns a CUDA error. */
cudaError_t fp32_launch_chunk(const Scn32* d_scn, int nscn, const int4* d_work, const int* class_first,
                              const int* class_n, Part32* d_part, void* d_ctl, int niter, const int* grid,
                              cudaStream_t s);
/* CTAs of class k's persistent kernel one SM holds */
int fp32_blocks_per_sm(int k);
void fp32_launch_prime(const Scn32* d_scn, int nscn, cudaStream_t s);
/* volume and CFL speed of one scenario into d_out[0..1]; d_out holds
 * fp32_volume_scratch_bytes() (the partials follow the two results) */
void fp32_launch_volume(const Scn32* d_scn, int iscn, const Scn32& host_scn, double* d_out, cudaStream_t s);
size_t fp32_volume_scratch_bytes();
/* boundary-discharge sample of one scenario (device descriptor d_scn_one):
 * faces holds (raster cell r*cols+c, side) pairs; q and vel_prev nfaces
 * doubles on the device */
void fp32_launch_couple(const Scn32* d_scn_one, int nfaces, const int* faces, int lagged, int initial, double th,
                        double* vel_prev, double* q, cudaStream_t s);
size_t fp32_smem_bytes();
int fp32_configure_kernels();

} // namespace sw2d
#endif
