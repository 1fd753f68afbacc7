/* Test infrastructure only: CPU oracle of SW2D's explicit 2-D overland step.
 *
 * A plain-C restatement of the reference's algorithm, SW2D-EFDC.cu:
 *   flux          :97-353   x/y face discharges (dry bed 1 & 2, gravity,
 *                           upwind convection, semi-implicit Manning)
 *   continuity    :602-664  depth update with rain/source/evaporation terms
 *   treat_error   :695-725  zero the outward faces of near-dry cells
 *   hm_hn         :362-398, uu1_vv1 :404-452, uu_vv :458-483, uua_vva :489-522
 *   forward       :670-693  time-level copy (here: the state is (h, qx, qy))
 *   stream_flow   :525-554, evaporation_load :588-600 (forcing interpolation)
 *   time loop     :4798-4878
 * plus the extensions the reference lacks: CFL step length, FP64 volume
 * ledger, a free-overfall south outlet, per-cell Manning n and rain weight.
 *
 * Layout: every field lives on a grid with a 2-cell halo of inactive, dry,
 * zero-flux cells, so the reference's raster-edge rules (zero faces on the
 * edge and next to NODATA) become one rule: a face is closed unless both of
 * its cells are active.  The two places where the reference's edge rule is
 * not the inactive-neighbour rule are kept explicitly: no cross-convection
 * term for x faces in column 0 (:184-186) and for y faces in row 0 (:280-284).
 *
 * math = ORC_MATH_LIBM evaluates every expression exactly as the reference
 * does (libm pow, IEEE divisions): it is the pinned restatement.
 * math = ORC_MATH_DEVICE swaps in the helpers of sw2d_math.h that the CUDA
 * FP64 kernels use (friction pow as a product, constant divisions by
 * reciprocal + residual), so the GPU result can be compared bit for bit.
 * Compile with -ffp-contract=off.
 */
#include "sw2d_oracle.h"
#include "sw2d_math.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define H 2

struct orc_state {
    orc_config c;
    int R, C, P;           /* rows, cols, pitch (cols + 2H) */
    double *z, *h, *qx, *qy, *uu1, *vv1;
    double *fx, *fy, *hs, *hn;
    double *nman;          /* per-cell Manning n or NULL */
    float *rw;             /* per-cell rain weight or NULL */
    unsigned char* act;
    int* srcmap;           /* per-cell source index or -1 */
    double* rain;          /* nrain + 2 (zero tail) */
    double* evap;          /* nevap + 2 or NULL */
    double* srcq;          /* (nq + 2) * nsrc */
    double t;
    long long iters;
    double dt2_next;       /* CFL: length of the next iteration */
    orc_ledger L;
    double* out_t;
    double* out_q;
    long long out_n, out_cap;
};

static inline size_t IX(const orc_state* s, int r, int c) {
    return (size_t)(r + H) * s->P + (size_t)(c + H);
}

/* ---------------- forcing: SW2D-EFDC.cu:525-554 and :588-600 ------------- */

/* Value of a series (entries per interval dts) at time `time`, in the
 * series' own unit.  Reference mode keeps the ramp for time <= 1 and the
 * interpolation exactly as written (it divides where linear interpolation
 * would multiply, SW2D-EFDC.cu:551). */
static double series_at(const double* v, int n, double dts, double time, int mode) {
    double r;
    int it;
    if (mode == ORC_RAIN_REFERENCE) {
        if (time <= 1.00) {
            r = v[0] * time;
        } else {
            it = sw2d_series_index(time, dts, n); /* past the series: zero tail */
            r = v[it] + (v[it + 1] - v[it]) / (dts * (time - dts * (it)));
        }
    } else if (mode == ORC_RAIN_LINEAR) {
        it = sw2d_series_index(time, dts, n);
        r = v[it] + (v[it + 1] - v[it]) * ((time - dts * (it)) / dts);
    } else {
        it = sw2d_series_index(time, dts, n);
        r = v[it];
    }
    return r;
}

static double rain_rate(const orc_state* s, double time) {
    double rr = series_at(s->rain, s->c.nrain, s->c.dtrain, time, s->c.rain_mode);
    return rr / (s->c.dtrain * 1000.0); /* mm per dtrain -> m/s */
}

static double evap_rate(const orc_state* s, double time) {
    if (!s->evap) return 0.0;
    double ev = series_at(s->evap, s->c.nevap, s->c.dtrain, time, s->c.rain_mode);
    return ev / (s->c.dtrain * 1000.0);
}

static void source_rates(const orc_state* s, double time, double* ql) {
    for (int i = 0; i < s->c.nsrc; i++) {
        double q;
        if (s->c.rain_mode == ORC_RAIN_REFERENCE) {
            if (time <= 1.00) {
                q = s->srcq[i] * time;
            } else {
                const int it = sw2d_series_index(time, s->c.dtoq, s->c.nq);
                q = s->srcq[(size_t)it * s->c.nsrc + i] +
                    (s->srcq[(size_t)(it + 1) * s->c.nsrc + i] - s->srcq[(size_t)it * s->c.nsrc + i]) /
                        (s->c.dtoq * (time - s->c.dtoq * (it)));
            }
        } else {
            const int it = sw2d_series_index(time, s->c.dtoq, s->c.nq);
            double a = s->srcq[(size_t)it * s->c.nsrc + i];
            if (s->c.rain_mode == ORC_RAIN_LINEAR) {
                double b = s->srcq[(size_t)(it + 1) * s->c.nsrc + i];
                q = a + (b - a) * ((time - s->c.dtoq * (it)) / s->c.dtoq);
            } else {
                q = a;
            }
        }
        ql[i] = q / (s->c.dx * s->c.dy); /* m3/s -> m/s */
    }
}

/* ---------------- flux: SW2D-EFDC.cu:97-353 ------------------------------ */

static inline double friction(const orc_state* s, double nf, double sq, double hm) {
    /* SW2D-EFDC.cu:193-198 (x) and :310-315 (y) */
    const double gg = s->c.g;
    if (hm <= s->c.th) return 0.00;
    if (s->c.math == ORC_MATH_LIBM) {
        double expx = pow((double)(hm), (double)(1.3333330));
        return gg * nf * nf * sq / expx;
    }
    return (gg * nf * nf * sq) * sw2d_rpow_manning(hm);
}

static inline double face_n(const orc_state* s, size_t a, size_t b) {
    if (!s->nman) return s->c.manning;
    return 0.50 * (s->nman[a] + s->nman[b]);
}

/* Discharge on the x face between cell (r-1, c) ("w", upstream row) and
 * (r, c) ("e"); positive towards increasing row (south). */
static double flux_x(const orc_state* s, int r, int c, double dt2, double dt2dx, double dt2dy) {
    const double th = s->c.th, gg = s->c.g;
    const int P = s->P;
    size_t e = IX(s, r, c), w = e - P;
    const double *h = s->h, *z = s->z, *umo = s->qx, *uu1 = s->uu1, *vv1 = s->vv1;

    if (r == s->R && s->c.outflow_south) {
        /* free overfall through the south edge: the reference's dry-bed
         * weir discharge 0.544 h sqrt(g h) of SW2D-EFDC.cu:131 */
        if (s->act[w] && h[w] > th) return 0.5440 * h[w] * sqrt(gg * h[w]);
        return 0;
    }
    if (!s->act[e] || !s->act[w]) return 0;                         /* :115-116, :112 */
    if (!((h[w] > th) || (h[e] > th))) return 0;                    /* :117 */

    double hhe = h[e] + z[e];
    double hhw = h[w] + z[w];
    double hhep = h[e] - th;
    double hhwp = h[w] - th;
    if (hhe < z[w]) {                                              /* :129-136 */
        if (h[w] > th) return 0.5440 * h[w] * sqrt(gg * h[w]);
        return 0;
    } else if (hhw < z[e]) {                                       /* :137-144 */
        if (h[e] > th) return -0.544 * h[e] * sqrt(gg * h[e]);
        return 0;
    } else if (hhep * hhwp < 0) {                                  /* :148-159 */
        if ((h[e] > 0) || (h[w] > 0)) {
            double hhan = hhep - hhwp;
            double sgnm = copysign(1.0, hhan); /* hhan / |hhan|, hhan != 0 here */
            double hh3 = fmax(hhe, hhw) - fmax(z[e], z[w]);
            return -sgnm * 0.350 * hh3 * sqrt(2.00 * gg * hh3);
        }
        return 0;
    }
    double hm = 0.50 * (h[e] + h[w]);                               /* :373-374 */
    /* gravity :165 */
    double u13 = gg * hm * dt2dx * (hhe - h[w] - z[w]);
    /* convection along x :171-175 */
    double u11uur = 0.50 * (uu1[e + P] + uu1[e]);
    double u11uul = 0.50 * (uu1[e] + uu1[w]);
    double umr = u11uur * (umo[e + P] + umo[e]) * 0.50 + fabs(u11uur) * (umo[e] - umo[e + P]) * 0.50;
    double uml = u11uul * (umo[e] + umo[w]) * 0.50 + fabs(u11uul) * (umo[w] - umo[e]) * 0.50;
    double u11 = dt2dx * (umr - uml);
    /* convection along y :177-189; none in column 0 */
    double u12;
    if (c == 0) {
        u12 = 0;
    } else {
        double u12vvu = 0.50 * (vv1[e + 1] + vv1[w + 1]);
        double u12vvd = 0.50 * (vv1[e] + vv1[w]);
        double umu = u12vvu * (umo[e + 1] + umo[e]) * 0.50 + fabs(u12vvu) * (umo[e] - umo[e + 1]) * 0.50;
        double umd = u12vvd * (umo[e - 1] + umo[e]) * 0.50 + fabs(u12vvd) * (umo[e - 1] - umo[e]) * 0.50;
        u12 = dt2dy * (umu - umd);
    }
    /* friction :193-198, with vva from uua_vva :502-503 */
    double vva = 0.250 * (vv1[e] + vv1[e + 1] + vv1[w] + vv1[w + 1]);
    double sqx = sqrt(uu1[e] * uu1[e] + vva * vva);
    double ram = friction(s, face_n(s, e, w), sqx, hm);
    /* :202 */
    return ((1.00 - dt2 * ram * 0.50) * umo[e] + (-u11 - u12 - u13)) / (1.00 + dt2 * ram * 0.50);
}

/* Discharge on the y face between cell (r, c-1) ("s") and (r, c) ("n");
 * positive towards increasing column (east). */
static double flux_y(const orc_state* s, int r, int c, double dt2, double dt2dx, double dt2dy) {
    const double th = s->c.th, gg = s->c.g;
    const int P = s->P;
    size_t n = IX(s, r, c), so = n - 1;
    const double *h = s->h, *z = s->z, *vno = s->qy, *uu1 = s->uu1, *vv1 = s->vv1;

    if (!s->act[n] || !s->act[so]) return 0;                        /* :231-233 */
    if (!((h[so] > th) || (h[n] > th))) return 0;                   /* :234 */

    double hhn = h[n] + z[n];
    double hhs = h[so] + z[so];
    double hhnp = h[n] - th;
    double hhsp = h[so] - th;
    if (hhn < z[so]) {                                             /* :246-253 */
        if (h[so] > th) return 0.5440 * h[so] * sqrt(gg * h[so]);
        return 0;
    } else if (hhs < z[n]) {                                       /* :254-261 */
        if (h[n] > th) return -0.544 * h[n] * sqrt(gg * h[n]);
        return 0;
    } else if (hhnp * hhsp < 0) {                                  /* :265-276 */
        if ((h[n] > 0) || (h[so] > 0)) {
            double hhan = hhnp - hhsp;
            double sgnm = copysign(1.0, hhan);
            double hh3 = fmax(hhn, hhs) - fmax(z[n], z[so]);
            return -sgnm * 0.350 * hh3 * sqrt(2.00 * gg * hh3);
        }
        return 0;
    }
    double hnf = 0.50 * (h[n] + h[so]);                             /* :374-376 */
    /* gravity :282 */
    double v13 = gg * hnf * dt2dy * (hhn - h[so] - z[so]);
    /* convection along x :288-300; none in row 0 */
    double v11;
    if (r == 0) {
        v11 = 0;
    } else {
        double v11uur = 0.50 * (uu1[n + P] + uu1[n + P - 1]);
        double v11uul = 0.50 * (uu1[n] + uu1[n - 1]);
        double vnr = v11uur * (vno[n + P] + vno[n]) * 0.50 + fabs(v11uur) * (vno[n] - vno[n + P]) * 0.50;
        double vnl = v11uul * (vno[n] + vno[n - P]) * 0.50 + fabs(v11uul) * (vno[n - P] - vno[n]) * 0.50;
        v11 = dt2dx * (vnr - vnl);
    }
    /* convection along y :302-306 */
    double v12vvu = 0.50 * (vv1[n + 1] + vv1[n]);
    double v12vvd = 0.50 * (vv1[n] + vv1[n - 1]);
    double vnu = v12vvu * (vno[n + 1] + vno[n]) * 0.50 + fabs(v12vvu) * (vno[n] - vno[n + 1]) * 0.50;
    double vnd = v12vvd * (vno[n - 1] + vno[n]) * 0.50 + fabs(v12vvd) * (vno[n - 1] - vno[n]) * 0.50;
    double v12 = dt2dy * (vnu - vnd);
    /* friction :310-315, with uua from uua_vva :500-501 */
    double uua = 0.250 * (uu1[n] + uu1[n + P] + uu1[n - 1] + uu1[n + P - 1]);
    double sqy = sqrt(uua * uua + vv1[n] * vv1[n]);
    double ram = friction(s, face_n(s, n, so), sqy, hnf);
    /* :319 */
    return ((1.00 - dt2 * ram * 0.50) * vno[n] + (-v11 - v12 - v13)) / (1.00 + dt2 * ram * 0.50);
}

/* ---------------- continuity: SW2D-EFDC.cu:602-664 ----------------------- */

static inline double cdiv(const orc_state* s, double a, double d) {
    if (s->c.math == ORC_MATH_LIBM) return a / d;
    return sw2d_div_const(a, d, 1.0 / d);
}

/* Depth from ho and face discharges fx/fy; *raw receives the value before the
 * max(h, 0) clamp (for the volume ledger). */
static inline double continuity_cell(const orc_state* s, size_t i, const double* fx,
                                     const double* fy, double dt2, double rr, double ev,
                                     const double* ql, double* raw) {
    const int P = s->P;
    double pct, evapo;
    double ho = s->h[i];
    if (ho > s->c.ev_wl_min) {                                     /* :626-633 */
        pct = 1.00 - s->c.frac_lwl;
        evapo = ev;
    } else {
        pct = 1.00 - (s->c.frac_int + s->c.frac_inf);
        evapo = 0.000;
    }
    double rcell = s->rw ? rr * (double)s->rw[i] : rr;
    double qli = (s->srcmap[i] >= 0) ? ql[s->srcmap[i]] : 0.0;
    double hnew = ho - dt2 * (cdiv(s, fx[i + P] - fx[i], s->c.dx) + cdiv(s, fy[i + 1] - fy[i], s->c.dy) -
                              qli - rcell * pct + evapo);          /* :653 */
    *raw = hnew;
    hnew = fmax(hnew, 0.00);                                       /* :656 */
    if (!s->act[i]) hnew = 0.00;                                   /* :657-659 */
    return hnew;
}

/* ---------------- setup ------------------------------------------------- */

static void* zalloc(size_t n) { return calloc(n ? n : 1, 1); }

static void update_face_velocities(orc_state* s);
static double cfl_speed(const orc_state* s);

orc_state* orc_create(const orc_config* cfg, const double* dem, const double* h0,
                      const double* manning, const float* rain_w, const double* rain,
                      const double* evap, const int* src_cell, const double* src_q) {
    orc_state* s = (orc_state*)zalloc(sizeof(orc_state));
    s->c = *cfg;
    s->R = cfg->rows;
    s->C = cfg->cols;
    s->P = cfg->cols + 2 * H;
    size_t n = (size_t)(s->R + 2 * H) * s->P;
    s->z = (double*)zalloc(n * sizeof(double));
    s->h = (double*)zalloc(n * sizeof(double));
    s->qx = (double*)zalloc(n * sizeof(double));
    s->qy = (double*)zalloc(n * sizeof(double));
    s->uu1 = (double*)zalloc(n * sizeof(double));
    s->vv1 = (double*)zalloc(n * sizeof(double));
    s->fx = (double*)zalloc(n * sizeof(double));
    s->fy = (double*)zalloc(n * sizeof(double));
    s->hs = (double*)zalloc(n * sizeof(double));
    s->hn = (double*)zalloc(n * sizeof(double));
    s->act = (unsigned char*)zalloc(n);
    s->srcmap = (int*)zalloc(n * sizeof(int));
    for (size_t i = 0; i < n; i++) s->srcmap[i] = -1;
    if (manning) s->nman = (double*)zalloc(n * sizeof(double));
    if (rain_w) s->rw = (float*)zalloc(n * sizeof(float));
    for (int r = 0; r < s->R; r++)
        for (int c = 0; c < s->C; c++) {
            size_t i = IX(s, r, c), k = (size_t)r * s->C + c;
            s->z[i] = dem[k];
            s->act[i] = (dem[k] != cfg->nodata);                   /* init_inf :37-42 */
            s->h[i] = s->act[i] ? h0[k] : 0.0;
            if (s->nman) s->nman[i] = manning[k];
            if (s->rw) s->rw[i] = rain_w[k];
        }
    s->rain = (double*)zalloc((size_t)(cfg->nrain + 2) * sizeof(double));
    if (rain && cfg->nrain > 0) memcpy(s->rain, rain, (size_t)cfg->nrain * sizeof(double));
    if (evap && cfg->nevap > 0) {
        s->evap = (double*)zalloc((size_t)(cfg->nevap + 2) * sizeof(double));
        memcpy(s->evap, evap, (size_t)cfg->nevap * sizeof(double));
    }
    int nsrc = cfg->nsrc > 0 ? cfg->nsrc : 0;
    s->srcq = (double*)zalloc((size_t)(cfg->nq + 2) * (nsrc ? nsrc : 1) * sizeof(double));
    if (nsrc) {
        memcpy(s->srcq, src_q, (size_t)cfg->nq * nsrc * sizeof(double));
        for (int i = 0; i < nsrc; i++) {
            int k = src_cell[i];
            int r = k / s->C, c = k % s->C;
            if (r >= 0 && r < s->R) s->srcmap[IX(s, r, c)] = i;
        }
    }
    s->t = cfg->t0;
    double v0 = 0;
    for (int r = 0; r < s->R; r++)
        for (int c = 0; c < s->C; c++) v0 += s->h[IX(s, r, c)];
    s->L.volume = s->L.volume0 = v0 * cfg->dx * cfg->dy;
    update_face_velocities(s);
    if (cfg->dt_mode == ORC_DT_CFL) {
        s->L.s_max = cfl_speed(s);
        s->dt2_next = s->L.s_max > 0 ? fmin(cfg->dt_max, cfg->cfl / s->L.s_max) : cfg->dt_max;
    }
    s->out_cap = 1024;
    s->out_t = (double*)malloc(s->out_cap * sizeof(double));
    s->out_q = (double*)malloc(s->out_cap * sizeof(double));
    return s;
}

void orc_destroy(orc_state* s) {
    if (!s) return;
    free(s->z); free(s->h); free(s->qx); free(s->qy); free(s->uu1); free(s->vv1);
    free(s->fx); free(s->fy); free(s->hs); free(s->hn); free(s->act); free(s->srcmap);
    free(s->nman); free(s->rw); free(s->rain); free(s->evap); free(s->srcq);
    free(s->out_t); free(s->out_q);
    free(s);
}

/* ---------------- diagnostics: SW2D-EFDC.cu:362-452 ---------------------- */

/* uu1 = qx / hm on x faces and vv1 = qy / hn on y faces, from the current
 * (h, qx, qy); hm on the north wall is the first row's depth and on the
 * south edge the last row's (:380-385), hn likewise on the west wall. */
static void update_face_velocities(orc_state* s) {
    const double th = s->c.th;
    const int P = s->P;
#pragma omp parallel for num_threads(s->c.nthreads > 0 ? s->c.nthreads : 1) schedule(static)
    for (int r = 0; r <= s->R; r++) {
        for (int c = 0; c <= s->C; c++) {
            size_t i = IX(s, r, c);
            if (c < s->C) {
                double hm;
                if (r == 0) hm = s->h[i];
                else if (r == s->R) hm = s->h[i - P];
                else hm = 0.50 * (s->h[i] + s->h[i - P]);
                s->uu1[i] = (hm >= th) ? s->qx[i] / hm : 0.00;     /* :414-419 */
            }
            if (r < s->R) {
                double hn;
                if (c == 0) hn = s->h[i];
                else if (c == s->C) hn = s->h[i - 1];
                else hn = 0.50 * (s->h[i] + s->h[i - 1]);
                s->vv1[i] = (hn >= th) ? s->qy[i] / hn : 0.0;      /* :421-426 */
            }
        }
    }
}

/* CFL speed of the state (h, qx, qy) with its face velocities uu1, vv1:
 *     S = max over x faces of (|uu1| + sqrt(g hm)) / dx
 *       + max over y faces of (|vv1| + sqrt(g hn)) / dy,
 * over faces whose two cells are active and whose mean depth is >= th.
 * An iteration's length is min(dt_max, cfl / S) with S of the state the
 * PREVIOUS iteration started from (the first two iterations use the initial
 * state), so the GPU can reduce S while it computes that iteration.  The
 * reference has no CFL control (its dt is fixed, SW2D-EFDC.cu:3770-3771). */
static double cfl_speed(const orc_state* s) {
    const double th = s->c.th, g = s->c.g;
    const double rdx = 1.0 / s->c.dx, rdy = 1.0 / s->c.dy;
    const int P = s->P;
    double mx = 0.0, my = 0.0;
    for (int r = 0; r < s->R; r++)
        for (int c = 0; c < s->C; c++) {
            size_t i = IX(s, r, c);
            if (!s->act[i]) continue;
            if (r > 0 && s->act[i - P]) {
                double hm = 0.50 * (s->h[i] + s->h[i - P]);
                if (hm >= th) {
                    double sp = (fabs(s->uu1[i]) + sqrt(g * hm)) * rdx;
                    if (sp > mx) mx = sp;
                }
            }
            if (c > 0 && s->act[i - 1]) {
                double hn = 0.50 * (s->h[i] + s->h[i - 1]);
                if (hn >= th) {
                    double sp = (fabs(s->vv1[i]) + sqrt(g * hn)) * rdy;
                    if (sp > my) my = sp;
                }
            }
        }
    return mx + my;
}

/* ---------------- one iteration: SW2D-EFDC.cu:4808-4877 ------------------ */

int orc_step(orc_state* s, double t_end) {
    const int P = s->P, R = s->R, C = s->C;
    const double th = s->c.th;
    double dt2, t_a, t_b, t_next;
    if (s->c.dt_mode == ORC_DT_FIXED) {
        double dt = s->c.dt;
        if (!(s->t + dt <= t_end)) return 0;                       /* :4798 */
        dt2 = 2.00 * dt;
        t_a = s->t;
        t_b = s->t + dt;                                           /* :4838 */
        t_next = t_b + dt;                                         /* :4876 */
    } else {
        if (!(s->t < t_end)) return 0;
        dt2 = s->dt2_next;
        if (s->t + dt2 > t_end) dt2 = t_end - s->t;
        t_a = s->t;
        t_b = s->t + 0.5 * dt2;
        t_next = s->t + dt2;
    }
    const double dt2dx = dt2 / s->c.dx, dt2dy = dt2 / s->c.dy;
    const int nt = s->c.nthreads > 0 ? s->c.nthreads : 1;
    const double s_entering = (s->c.dt_mode == ORC_DT_CFL) ? cfl_speed(s) : 0.0;

    /* 1. flux (:4810) */
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int r = 0; r <= R; r++)
        for (int c = 0; c <= C; c++) {
            size_t i = IX(s, r, c);
            s->fx[i] = (c < C) ? flux_x(s, r, c, dt2, dt2dx, dt2dy) : 0.0;
            s->fy[i] = (r < R) ? flux_y(s, r, c, dt2, dt2dx, dt2dy) : 0.0;
        }

    double ql1[64], ql2[64];
    double* q1 = s->c.nsrc > 64 ? (double*)malloc(sizeof(double) * s->c.nsrc) : ql1;
    double* q2 = s->c.nsrc > 64 ? (double*)malloc(sizeof(double) * s->c.nsrc) : ql2;
    source_rates(s, t_a, q1);
    source_rates(s, t_b, q2);
    const double rr1 = rain_rate(s, t_a), rr2 = rain_rate(s, t_b);
    const double ev1 = evap_rate(s, t_a), ev2 = evap_rate(s, t_b);

    /* 2. provisional depth (:4829) */
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int r = 0; r < R; r++)
        for (int c = 0; c < C; c++) {
            size_t i = IX(s, r, c);
            double raw;
            s->hs[i] = continuity_cell(s, i, s->fx, s->fy, dt2, rr1, ev1, q1, &raw);
        }

    /* 3. treat_error (:4835) as a per-face rule: a face carrying water out of
     * an active cell whose provisional depth is below th is closed. */
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int r = 0; r <= R; r++)
        for (int c = 0; c <= C; c++) {
            size_t i = IX(s, r, c);
            if (c < C) {
                double f = s->fx[i];
                if (f > 0 && s->act[i - P] && s->hs[i - P] < th) s->fx[i] = 0; /* :706-708 */
                if (f < 0 && r < R && s->act[i] && s->hs[i] < th) s->fx[i] = 0.00; /* :710 */
            }
            if (r < R) {
                double f = s->fy[i];
                if (f > 0 && s->act[i - 1] && s->hs[i - 1] < th) s->fy[i] = 0; /* :712-714 */
                if (f < 0 && c < C && s->act[i] && s->hs[i] < th) s->fy[i] = 0; /* :716 */
            }
        }

    /* 4. final depth (:4854) with the ledger sums per row */
    double* rowsum = (double*)calloc((size_t)R * 4, sizeof(double));
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int r = 0; r < R; r++) {
        double vol = 0, rain = 0, clamp = 0, evap = 0;
        for (int c = 0; c < C; c++) {
            size_t i = IX(s, r, c);
            double raw;
            double hn = continuity_cell(s, i, s->fx, s->fy, dt2, rr2, ev2, q2, &raw);
            s->hn[i] = hn;
            if (s->act[i]) {
                double pct = (s->h[i] > s->c.ev_wl_min) ? 1.00 - s->c.frac_lwl
                                                        : 1.00 - (s->c.frac_int + s->c.frac_inf);
                double rcell = s->rw ? rr2 * (double)s->rw[i] : rr2;
                rain += rcell * pct;
                if (s->h[i] > s->c.ev_wl_min) evap += ev2;
                clamp += hn - raw;
                vol += hn;
            }
        }
        rowsum[4 * r + 0] = vol;
        rowsum[4 * r + 1] = rain;
        rowsum[4 * r + 2] = clamp;
        rowsum[4 * r + 3] = evap;
    }
    double vol = 0, rain = 0, clamp = 0, evap = 0, qout = 0, src = 0;
    for (int r = 0; r < R; r++) {
        vol += rowsum[4 * r + 0];
        rain += rowsum[4 * r + 1];
        clamp += rowsum[4 * r + 2];
        evap += rowsum[4 * r + 3];
    }
    free(rowsum);
    if (s->c.outflow_south)
        for (int c = 0; c < C; c++) qout += s->fx[IX(s, R, c)];
    for (int k = 0; k < s->c.nsrc; k++) src += q2[k];
    if (q1 != ql1) free(q1);
    if (q2 != ql2) free(q2);

    /* 5. new state (forward :4872): swap the new fields in */
    double* tmp;
    tmp = s->h; s->h = s->hn; s->hn = tmp;
    tmp = s->qx; s->qx = s->fx; s->fx = tmp;
    tmp = s->qy; s->qy = s->fy; s->fy = tmp;
    update_face_velocities(s);                                     /* :4860-4862 */

    const double area = s->c.dx * s->c.dy;
    s->L.volume = vol * area;
    s->L.rain_in += dt2 * rain * area;
    s->L.clamp_gain += clamp * area;
    s->L.evap_out += dt2 * evap * area;
    s->L.source_in += dt2 * src * area;
    s->L.q_out = qout * s->c.dy;
    s->L.outflow += dt2 * s->L.q_out;
    s->L.dt2_last = dt2;
    s->t = t_next;
    s->iters++;
    if (s->c.dt_mode == ORC_DT_CFL) {
        s->L.s_max = s_entering;
        s->dt2_next = s->L.s_max > 0 ? fmin(s->c.dt_max, s->c.cfl / s->L.s_max) : s->c.dt_max;
    }
    if (s->out_n == s->out_cap) {
        s->out_cap *= 2;
        s->out_t = (double*)realloc(s->out_t, s->out_cap * sizeof(double));
        s->out_q = (double*)realloc(s->out_q, s->out_cap * sizeof(double));
    }
    s->out_t[s->out_n] = s->t;
    s->out_q[s->out_n] = s->L.q_out;
    s->out_n++;
    return 1;
}

long long orc_run(orc_state* s, double t_end, long long max_iters) {
    long long n = 0;
    while ((max_iters < 0 || n < max_iters) && orc_step(s, t_end)) n++;
    return n;
}

double orc_time(const orc_state* s) { return s->t; }
long long orc_iters(const orc_state* s) { return s->iters; }
void orc_ledger_get(const orc_state* s, orc_ledger* out) { *out = s->L; }
long long orc_outlet_count(const orc_state* s) { return s->out_n; }
void orc_outlet_get(const orc_state* s, double* t, double* q) {
    memcpy(t, s->out_t, (size_t)s->out_n * sizeof(double));
    memcpy(q, s->out_q, (size_t)s->out_n * sizeof(double));
}

void orc_get_fields(const orc_state* s, double* depth, double* qx, double* qy, double* uu,
                    double* vv, double* uua, double* vva) {
    const int R = s->R, C = s->C, P = s->P;
    const double th = s->c.th;
    for (int r = 0; r <= R; r++)
        for (int c = 0; c <= C; c++) {
            size_t i = IX(s, r, c);
            if (qx && c < C) qx[(size_t)r * C + c] = s->qx[i];
            if (qy && r < R) qy[(size_t)r * (C + 1) + c] = s->qy[i];
            if (r == R || c == C) continue;
            size_t k = (size_t)r * C + c;
            if (depth) depth[k] = s->h[i];
            if (uu || vv) { /* uu_vv :468-476 */
                double a = 0, b = 0;
                if (s->h[i] >= th) {
                    a = (s->uu1[i + P] + s->uu1[i]) / 2.00;
                    b = (s->vv1[i + 1] + s->vv1[i]) / 2.00;
                }
                if (uu) uu[k] = a;
                if (vv) vv[k] = b;
            }
            if (uua) /* uua_vva :499-510 */
                uua[k] = (c > 0) ? 0.250 * (s->uu1[i] + s->uu1[i + P] + s->uu1[i - 1] + s->uu1[i + P - 1])
                                 : 0.50 * (s->uu1[i] + s->uu1[i + P]);
            if (vva)
                vva[k] = (r > 0) ? 0.250 * (s->vv1[i] + s->vv1[i + 1] + s->vv1[i - P] + s->vv1[i - P + 1])
                                 : 0.50 * (s->vv1[i] + s->vv1[i + 1]);
        }
}

/* ---------------- coupling: SW2D-EFDC.cu:728-1067 ------------------------ */

enum { SIDE_N = 0, SIDE_S = 1, SIDE_E = 2, SIDE_W = 3 };

static int add_face(int* n, int max, int* side, int* ci, int* cj, int* cell, int sd, int i, int j, int p) {
    if (*n < max) {
        side[*n] = sd;
        ci[*n] = i;
        cj[*n] = j;
        cell[*n] = p;
    }
    (*n)++;
    return 0;
}

int orc_couple_faces(int rows, int cols, const int* mask, int max_faces, int* side, int* ci,
                     int* cj, int* cell) {
    int n = 0;
    for (int ini = 0; ini < rows; ini++) {            /* ini counts rows from the bottom */
        int base = rows * cols - (ini + 1) * cols;
        for (int inj = 0; inj < cols; inj++) {
            int p = base + inj;
            if (mask[p] == 1) continue;
            int S = 0, N = 0, E = 0, W = 0;
            if (ini > 0 && ini < rows - 1) {
                if (inj > 0 && inj < cols - 1) { S = N = E = W = 1; }
                else if (inj == cols - 1) { S = N = E = 1; }
                else if (inj == 0) { S = N = W = 1; }
            }
            if (inj > 0 && inj < cols - 1) {
                if (ini == 0) { S = E = W = 1; }
                else if (ini == rows - 1) { N = E = W = 1; }
            }
            if (S && mask[p] != mask[p - cols]) add_face(&n, max_faces, side, ci, cj, cell, SIDE_S, inj + 1, ini + 2, p);
            if (N && mask[p] != mask[p + cols]) add_face(&n, max_faces, side, ci, cj, cell, SIDE_N, inj + 1, ini, p);
            if (E && mask[p] != mask[p - 1]) add_face(&n, max_faces, side, ci, cj, cell, SIDE_E, inj, ini + 1, p);
            if (W && mask[p] != mask[p + 1]) add_face(&n, max_faces, side, ci, cj, cell, SIDE_W, inj + 2, ini + 1, p);
        }
    }
    return n;
}

void orc_couple_values(int rows, int cols, double dx, double dy, int nfaces, const int* side,
                       const int* cell, const double* h, const double* uua, const double* vva,
                       double* q) {
    (void)rows;
    (void)cols;
    for (int k = 0; k < nfaces; k++) {
        int p = cell[k];
        double v;
        switch (side[k]) {
        case SIDE_S: v = (uua[p] < 0) ? -uua[p] * h[p] * dx : 0.00; break;
        case SIDE_N: v = (uua[p] > 0) ? uua[p] * h[p] * dx : 0.00; break;
        case SIDE_E: v = (vva[p] < 0) ? -vva[p] * h[p] * dy : 0.00; break;
        default: v = (vva[p] > 0) ? vva[p] * h[p] * dy : 0.00; break;
        }
        q[k] = v;
    }
}
