/* Test infrastructure only: never linked into the product.
 *
 * Drives the reference's own SW2D kernels (SW2D-EFDC.cu:29-725, compiled
 * unmodified through ref_shim.h) with a host loop that restates the
 * reference's time loop SW2D-EFDC.cu:4798-4878 and its coupling sample at
 * output intervals SW2D-EFDC.cu:4880-4916.  Each "launch" is an OpenMP
 * parallel region in which every thread plays one block of one thread.
 *
 * Arrays are allocated with (rows+2)*cols entries instead of the reference's
 * N = rows*cols + cols/2 so that the reference's reads past N (flux at
 * SW2D-EFDC.cu:171-173 and :295-297, continuity at :653, uu_vv at :474,
 * uua_vva at :504) land in zero-filled memory: a wall with zero flux.  DEM
 * padding (the cols/2 values after the raster) is NODATA, i.e. inactive.
 */
#include "ref_shim.h"

thread_local ref_dim3 threadIdx = {0, 0, 0};
thread_local ref_dim3 blockIdx = {0, 0, 0};
ref_dim3 blockDim = {1, 1, 1};
ref_dim3 gridDim = {1, 1, 1};

#include "ref_kernels.inc"
#include "ref_case.h"

#include <vector>
#include <cstring>

#define REF_LAUNCH(kernel, ...)                                   \
    do {                                                          \
        _Pragma("omp parallel num_threads(gridDim.x)")            \
        {                                                         \
            blockIdx.x = (unsigned)omp_get_thread_num();          \
            threadIdx.x = 0;                                      \
            kernel(__VA_ARGS__);                                  \
        }                                                         \
    } while (0)

extern "C" {

int sw2dref_water_cells(int rows, int cols, const int* mask) {
    int n = 0;
    for (int i = 0; i < rows * cols; i++) n += (mask[i] == 1);
    return n;
}

int sw2dref_run(const sw2dref_case* c, sw2dref_out* o) {
    const int rows = c->rows, cols = c->cols;
    const int N = rows * cols + cols / 2;          /* SW2D-EFDC.cu:3997 */
    const size_t A = (size_t)(rows + 2) * cols;    /* allocation incl. zero tail */
    gridDim.x = (unsigned)(c->nthreads > 0 ? c->nthreads : 1);
    blockDim.x = 1;

    std::vector<double> baseo(A, c->nodata), h(A, 0.0), ho(A, 0.0), hm(A, 0.0), hn(A, 0.0),
        um(A, 0.0), umo(A, 0.0), uu(A, 0.0), uua(A, 0.0), uu1(A, 0.0), vn(A, 0.0), vno(A, 0.0),
        vv(A, 0.0), vva(A, 0.0), vv1(A, 0.0), ql(A, 0.0), h_init(A, 0.0);
    std::vector<int> inf(A, 0), infx(A, 0), infy(A, 0);
    for (int i = 0; i < rows * cols; i++) {
        baseo[i] = c->dem[i];
        h[i] = c->h0[i];
        h_init[i] = c->h0[i];
    }
    double th = 1.0e-4;                            /* SW2D-EFDC.cu:4644 */
    double rr = 0.0, ev = 0.0;
    const double gg = 9.80;                        /* SW2D-EFDC.cu:3977 */
    const double dt = c->dt, dt2 = 2.00 * dt;      /* SW2D-EFDC.cu:3976 */
    const double dx = c->cellsize, dy = c->cellsize;

    std::vector<double> rain(c->rain, c->rain + c->nrain);
    rain.resize(c->nrain + 2, 0.0);
    std::vector<double*> qq_rows(c->nqq + 2);
    std::vector<double> qq_store((size_t)(c->nqq + 2) * (c->nst > 0 ? c->nst : 1), 0.0);
    for (int j = 0; j < c->nqq + 2; j++) {
        qq_rows[j] = &qq_store[(size_t)j * (c->nst > 0 ? c->nst : 1)];
        if (j < c->nqq)
            for (int i = 0; i < c->nst; i++) qq_rows[j][i] = c->qq[(size_t)j * c->nst + i];
    }
    std::vector<double> brx(c->brx, c->brx + c->nst), bry(c->bry, c->bry + c->nst);

    std::vector<double> evapo(c->nrain + 2, 0.0);
    if (c->evaporation_on) {
        std::vector<double> T(c->temp, c->temp + c->nrain), Rg(c->rad, c->rad + c->nrain),
            Rs(c->nrain), pw(c->nrain), lv(c->nrain);
        REF_LAUNCH(gpu_evaporation_calc, c->albedo, T.data(), Rg.data(), Rs.data(), pw.data(),
                   lv.data(), evapo.data(), c->dtrain, c->nrain);
    }

    /* coupling state, SW2D-EFDC.cu:4374-4400 */
    const bool couple = c->mask != NULL && c->lkout > 0;
    int water_cells = 0;
    std::vector<int> mask;
    std::vector<int*> bcp[4];
    std::vector<double*> valp[4];
    std::vector<int> bcs[4];
    std::vector<double> vals[4];
    std::vector<double> h_uua(A, 0.0), h_vva(A, 0.0), h_h(A, 0.0);
    int nqs = 0;
    if (couple) {
        mask.assign(A, 0);
        for (int i = 0; i < rows * cols; i++) mask[i] = c->mask[i];
        water_cells = sw2dref_water_cells(rows, cols, c->mask);
        for (int s = 0; s < 4; s++) {
            bcs[s].assign((size_t)(water_cells + 1) * 3, 0);
            vals[s].assign((size_t)(c->max_samples + 1) * (water_cells + 1), 0.0);
            bcp[s].resize(water_cells + 1);
            valp[s].resize(c->max_samples + 1);
            for (int i = 0; i <= water_cells; i++) bcp[s][i] = &bcs[s][(size_t)i * 3];
            for (int t = 0; t <= c->max_samples; t++) valp[s][t] = &vals[s][(size_t)t * (water_cells + 1)];
        }
    }

    /* SW2D-EFDC.cu:4763-4766 */
    REF_LAUNCH(init_inf, rows, cols, ho.data(), h.data(), inf.data(), baseo.data(), N, c->nodata);
    REF_LAUNCH(initiald, rows, cols, h.data(), infx.data(), infy.data(), inf.data(), hm.data(),
               hn.data(), baseo.data(), N, c->nodata);

    double time = c->time0;
    int mstep = 0, tq = -1, out0 = -1;
    long long iters = 0;
    double wall0 = omp_get_wtime();
    while (time + dt <= c->timmax) {               /* SW2D-EFDC.cu:4798 */
        if (iters == c->warm_iters) wall0 = omp_get_wtime();
        out0 = out0 + 1;
        REF_LAUNCH(flux, &th, gg, c->manning, inf.data(), h.data(), infx.data(), infy.data(),
                   baseo.data(), um.data(), hm.data(), uu1.data(), umo.data(), vv1.data(),
                   vva.data(), vn.data(), hn.data(), vno.data(), uua.data(), ho.data(), N, cols,
                   rows, dx, dy, dt2);
        stream_flow(cols, rows, c->xcoor_c, c->ycoor_c, time, c->dtrain, rain.data(),
                    qq_rows.data(), ql.data(), c->dtoq, brx.data(), bry.data(), dx, dy, c->nst, &rr);
        if (c->evaporation_on) evaporation_load(time, c->dtrain, evapo.data(), &ev);
        REF_LAUNCH(continuity, dt2, cols, rows, dx, dy, &rr, &ev, ql.data(), h.data(), ho.data(),
                   um.data(), vn.data(), c->frac_int, c->frac_inf, c->frac_lwl, c->ev_wl_min,
                   inf.data(), N);
        REF_LAUNCH(treat_error, cols, rows, &th, inf.data(), um.data(), vn.data(), h.data(), N);
        time = time + dt;
        mstep = mstep + 1;
        stream_flow(cols, rows, c->xcoor_c, c->ycoor_c, time, c->dtrain, rain.data(),
                    qq_rows.data(), ql.data(), c->dtoq, brx.data(), bry.data(), dx, dy, c->nst, &rr);
        if (c->evaporation_on) evaporation_load(time, c->dtrain, evapo.data(), &ev);
        REF_LAUNCH(continuity, dt2, cols, rows, dx, dy, &rr, &ev, ql.data(), h.data(), ho.data(),
                   um.data(), vn.data(), c->frac_int, c->frac_inf, c->frac_lwl, c->ev_wl_min,
                   inf.data(), N);
        REF_LAUNCH(hm_hn, hm.data(), hn.data(), h.data(), N, cols, rows);
        REF_LAUNCH(uu1_vv1, &th, hm.data(), hn.data(), uu1.data(), um.data(), vv1.data(), vn.data(),
                   N, cols, rows);
        REF_LAUNCH(uu_vv, &th, h.data(), uu1.data(), vv1.data(), uu.data(), vv.data(), N, cols);
        REF_LAUNCH(uua_vva, uu1.data(), vv1.data(), uua.data(), vva.data(), N, cols, rows);
        REF_LAUNCH(forward, cols, rows, umo.data(), um.data(), vno.data(), vn.data(), ho.data(),
                   h.data(), N);
        time = time + dt;
        mstep = mstep + 1;
        iters++;

        /* SW2D-EFDC.cu:4880-4916: coupling sample, velocities copied after the call */
        if (couple && ((mstep % c->lkout == 0) || (out0 == 0))) {
            tq = tq + 1;
            if (tq > c->max_samples) return -2;
            double efdc_time = mstep * dt / c->efdc_basetime;
            int q = 0;
            if (tq == 0) {
                couple_BC_efdc(1, cols, rows, dx, dy, &q, bcp[0].data(), bcp[1].data(), bcp[2].data(),
                               bcp[3].data(), valp[0].data(), valp[1].data(), valp[2].data(),
                               valp[3].data(), mask.data(), h_init.data(), h_vva.data(), h_uua.data(),
                               tq, 0.0000);
            } else {
                std::memcpy(h_h.data(), h.data(), sizeof(double) * N);
                couple_BC_efdc(1, cols, rows, dx, dy, &q, bcp[0].data(), bcp[1].data(), bcp[2].data(),
                               bcp[3].data(), valp[0].data(), valp[1].data(), valp[2].data(),
                               valp[3].data(), mask.data(), h_h.data(), h_vva.data(), h_uua.data(),
                               tq, efdc_time);
            }
            nqs = q;
            std::memcpy(h_uua.data(), uua.data(), sizeof(double) * N);
            std::memcpy(h_vva.data(), vva.data(), sizeof(double) * N);
        }
    }

    o->loop_seconds = omp_get_wtime() - wall0;
    double* outs[7] = {o->h, o->um, o->vn, o->uu, o->vv, o->uua, o->vva};
    const std::vector<double>* srcs[7] = {&h, &um, &vn, &uu, &vv, &uua, &vva};
    for (int k = 0; k < 7; k++)
        if (outs[k]) std::memcpy(outs[k], srcs[k]->data(), sizeof(double) * N);
    o->iters = iters;
    o->time = time;
    o->water_cells = water_cells;
    o->nqs = nqs;
    o->nsamples = tq + 1;
    if (couple) {
        for (int s = 0; s < 4; s++) {
            if (o->bc)
                std::memcpy(o->bc + (size_t)s * water_cells * 3, bcs[s].data(),
                            sizeof(int) * (size_t)water_cells * 3);
            if (o->val)
                std::memcpy(o->val + (size_t)s * c->max_samples * (water_cells + 1), vals[s].data(),
                            sizeof(double) * (size_t)c->max_samples * (water_cells + 1));
        }
    }
    return 0;
}

/* The reference's own QSER.INP writer (write_efdc_QSER, SW2D-EFDC.cu:2499-2610)
 * on the per-side arrays sw2dref_run returns: bc is 4 x water_cells x 3,
 * val is 4 x max_samples x (water_cells + 1); nsamples = tq + 1. */
int sw2dref_write_qser(const char* path, int type, int nlayers, const int* bc, const double* val, int water_cells,
                       int max_samples, double efdc_basetime, int nsamples) {
    std::vector<int> bcs[4];
    std::vector<double> vals[4];
    std::vector<int*> bcp[4];
    std::vector<double*> valp[4];
    for (int s = 0; s < 4; s++) {
        bcs[s].assign((size_t)(water_cells + 1) * 3, 0); /* zero row ends each side's list */
        std::memcpy(bcs[s].data(), bc + (size_t)s * water_cells * 3, sizeof(int) * (size_t)water_cells * 3);
        vals[s].assign(val + (size_t)s * max_samples * (water_cells + 1),
                       val + (size_t)(s + 1) * max_samples * (water_cells + 1));
        bcp[s].resize(water_cells + 1);
        valp[s].resize(max_samples);
        for (int i = 0; i <= water_cells; i++) bcp[s][i] = &bcs[s][(size_t)i * 3];
        for (int t = 0; t < max_samples; t++) valp[s][t] = &vals[s][(size_t)t * (water_cells + 1)];
    }
    write_efdc_QSER(path, type, nlayers, bcp[0].data(), bcp[1].data(), bcp[2].data(), bcp[3].data(),
                    valp[0].data(), valp[1].data(), valp[2].data(), valp[3].data(), efdc_basetime, nsamples - 1);
    return 0;
}

/* The reference's dye / temperature / salinity deck writers on the same
 * arrays: kind 'D' (write_efdc_DSER, concentration value[0]), 'T'
 * (write_efdc_TSER, the series value), 'S' (write_efdc_SSER, value[0]). */
int sw2dref_write_conc(const char* path, char kind, int type, int nlayers, const int* bc, const double* val,
                       int water_cells, int max_samples, double efdc_basetime, int nsamples, double* value) {
    std::vector<int> bcs[4];
    std::vector<int*> bcp[4];
    for (int s = 0; s < 4; s++) {
        bcs[s].assign((size_t)(water_cells + 1) * 3, 0);
        std::memcpy(bcs[s].data(), bc + (size_t)s * water_cells * 3, sizeof(int) * (size_t)water_cells * 3);
        bcp[s].resize(water_cells + 1);
        for (int i = 0; i <= water_cells; i++) bcp[s][i] = &bcs[s][(size_t)i * 3];
    }
    std::vector<double> north(val, val + (size_t)max_samples * (water_cells + 1));
    std::vector<double*> np(max_samples);
    for (int t = 0; t < max_samples; t++) np[t] = &north[(size_t)t * (water_cells + 1)];
    if (kind == 'D')
        write_efdc_DSER(path, type, nlayers, bcp[0].data(), bcp[1].data(), bcp[2].data(), bcp[3].data(), np.data(),
                        value[0], efdc_basetime, nsamples - 1);
    else if (kind == 'T')
        write_efdc_TSER(path, type, nlayers, bcp[0].data(), bcp[1].data(), bcp[2].data(), bcp[3].data(), np.data(),
                        value, efdc_basetime, nsamples - 1);
    else
        write_efdc_SSER(path, type, nlayers, bcp[0].data(), bcp[1].data(), bcp[2].data(), bcp[3].data(), np.data(),
                        value[0], efdc_basetime, nsamples - 1);
    return 0;
}

/* The reference's evaporation series (gpu_evaporation_calc,
 * SW2D-EFDC.cu:556-586) over n entries, on one host thread. */
int sw2dref_evaporation(int n, const double* temp, const double* rad, double albedo, double dtrain, double* out) {
    gridDim.x = 1;
    blockDim.x = 1;
    std::vector<double> T(temp, temp + n), Rg(rad, rad + n), Rs(n), pw(n), lv(n);
    REF_LAUNCH(gpu_evaporation_calc, albedo, T.data(), Rg.data(), Rs.data(), pw.data(), lv.data(), out, dtrain, n);
    return 0;
}

/* The reference's DEM pre-pass of a coupled run (lake_catchment_smooth,
 * SW2D-EFDC.cu:2766-2827), in place. */
int sw2dref_lake_smooth(int rows, int cols, int* mask, double* baseo) {
    lake_catchment_smooth(cols, rows, mask, baseo);
    return 0;
}

/* The reference's EFDC.INP configuration writer (write_efdc_CONFIG,
 * SW2D-EFDC.cu:1069-2025) on an existing EFDC.INP, with the face arrays of a
 * coupling run (4 sides x water_cells x 3, as sw2dref_run returns them) and
 * fixed values for the cards that do not depend on the faces. */
int sw2dref_write_config(const char* path, const int* bc, int water_cells, int nqs, int nlayers, int salt_on,
                         int temp_on, int dye_on) {
    std::vector<int> bcs[4];
    std::vector<int*> bcp[4];
    for (int s = 0; s < 4; s++) {
        bcs[s].assign((size_t)(water_cells + 1) * 3, 0);
        std::memcpy(bcs[s].data(), bc + (size_t)s * water_cells * 3, sizeof(int) * (size_t)water_cells * 3);
        bcp[s].resize(water_cells + 1);
        for (int i = 0; i <= water_cells; i++) bcp[s][i] = &bcs[s][(size_t)i * 3];
    }
    int nqsij = nqs;
    int lts_row[2] = {1, 1};
    int* lts[1] = {lts_row};
    write_efdc_CONFIG(path, &nqsij, nqs, bcp[0].data(), bcp[1].data(), bcp[2].data(), bcp[3].data(), nlayers,
                      /*ncols*/ 10, /*nrows*/ 10, water_cells, /*TCON*/ 3600.0, /*TBEGIN*/ 0.0, /*TREF*/ 3600.0,
                      /*NTC*/ 2, /*NTSPTC*/ 360, /*NTCPP*/ 2, /*NTCVB*/ 2, /*ISPPH*/ 1, /*NPPPH*/ 4, /*ISRPPH*/ 0,
                      /*IPPHXY*/ 0, /*ISVPH*/ 1, /*NPVPH*/ 4, /*ISRVPH*/ 0, /*IVPHXY*/ 0, /*ISTMSR*/ 1, /*MLTMSR*/ 1,
                      /*NBTMSR*/ 1, /*NSTMSR*/ 720, /*NWTMSR*/ 360, /*NTSSTSP*/ 1, /*TCTMSR*/ 1.0, /*nts_out*/ 1, lts,
                      /*NTSSSS*/ 1, /*MTSP*/ 1, /*MTSC*/ 1, /*MTSA*/ 0, /*MTSUE*/ 1, /*MTSUT*/ 1, /*MTSU*/ 0,
                      /*ZBRADJ*/ 0.0, /*ZBRCVRT*/ 1.0, /*HMIN*/ 0.1, /*HADJ*/ 0.0, /*HCVRT*/ 1.0, /*HDRY*/ 0.05,
                      /*HWET*/ 0.1, /*BELADJ*/ 0.0, /*BELCVRT*/ 1.0, /*NWSER*/ 0, /*NASER*/ 1, /*DX*/ 10.0,
                      /*DY*/ 10.0, dye_on, salt_on, temp_on, /*temp_opt*/ 1);
    return 0;
}

} /* extern "C" */
