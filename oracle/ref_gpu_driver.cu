/* Test infrastructure only: never linked into the product.
 *
 * Runs the reference's own SW2D kernels (SW2D-EFDC.cu:29-725, the extracted
 * range compiled unmodified by nvcc) on the GPU with the reference's launch
 * configuration and host loop (SW2D-EFDC.cu:4750-4758, :4798-4878): 1024
 * threads per block over N = rows*cols + cols/2 with grid-stride loops, a
 * device-wide synchronisation after every launch, and the point-source field
 * ql (N doubles) and the rain rate copied to the device twice per
 * iteration.  This is the "reference GPU" timing line; the fields it returns
 * let the tests check it against the CPU build of the same kernels.
 *
 * Arrays hold (rows+2)*cols entries instead of N, zero-filled (the DEM
 * padding NODATA), so that the reference's reads past N (SW2D-EFDC.cu:171-173,
 * :295-297, :653, :474, :504) stay inside the allocations and read the
 * zero-discharge wall they stand for; the same layout runs clean under
 * AddressSanitizer in the CPU build.  Coupling samples are not taken here.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "ref_kernels.inc"
#include "ref_case.h"

namespace {

struct DevBuf {
    double* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};
struct DevIBuf {
    int* p = nullptr;
    ~DevIBuf() {
        if (p) cudaFree(p);
    }
};

#define RCK(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            std::fprintf(stderr, "reference GPU driver: %s: %s\n", #call, cudaGetErrorString(e_)); \
            return -3;                                                              \
        }                                                                           \
    } while (0)

} // namespace

extern "C" {

int sw2dref_gpu_run(const sw2dref_case* c, sw2dref_out* o) {
    const int rows = c->rows, cols = c->cols;
    const int N = rows * cols + cols / 2;       /* SW2D-EFDC.cu:3997 */
    const size_t A = (size_t)(rows + 2) * cols; /* allocation incl. zero tail */
    const size_t B = A * sizeof(double);

    /* launch configuration, SW2D-EFDC.cu:4750-4758 */
    int maxThreadsPerBlock = 1024;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, 0) == cudaSuccess) maxThreadsPerBlock = prop.maxThreadsPerBlock;
    int threadsPerBlock, numBlocks;
    if (N < maxThreadsPerBlock) {
        threadsPerBlock = N;
        numBlocks = 1;
    } else {
        threadsPerBlock = maxThreadsPerBlock;
        numBlocks = (N + maxThreadsPerBlock - 1) / maxThreadsPerBlock;
    }

    std::vector<double> baseo(A, c->nodata), h(A, 0.0), ql(A, 0.0);
    for (int i = 0; i < rows * cols; i++) {
        baseo[i] = c->dem[i];
        h[i] = c->h0[i];
    }
    DevBuf d_baseo, d_h, d_ho, d_hm, d_hn, d_um, d_umo, d_uu, d_uua, d_uu1, d_vn, d_vno, d_vv, d_vva, d_vv1,
        d_ql, d_th, d_rr, d_Ev;
    DevIBuf d_inf, d_infx, d_infy;
    DevBuf* dbl[] = {&d_baseo, &d_h, &d_ho, &d_hm, &d_hn, &d_um, &d_umo, &d_uu,
                     &d_uua,   &d_uu1, &d_vn, &d_vno, &d_vv, &d_vva, &d_vv1, &d_ql};
    for (DevBuf* b : dbl) {
        RCK(cudaMalloc(&b->p, B));
        RCK(cudaMemset(b->p, 0, B));
    }
    DevIBuf* ints[] = {&d_inf, &d_infx, &d_infy};
    for (DevIBuf* b : ints) {
        RCK(cudaMalloc(&b->p, A * sizeof(int)));
        RCK(cudaMemset(b->p, 0, A * sizeof(int)));
    }
    RCK(cudaMalloc(&d_th.p, sizeof(double)));
    RCK(cudaMalloc(&d_rr.p, sizeof(double)));
    RCK(cudaMalloc(&d_Ev.p, sizeof(double)));
    double th = 1.0e-4; /* SW2D-EFDC.cu:4644 */
    double rr = 0.0, ev = 0.0;
    RCK(cudaMemcpy(d_th.p, &th, sizeof(double), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(d_Ev.p, &ev, sizeof(double), cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(d_baseo.p, baseo.data(), B, cudaMemcpyHostToDevice));
    RCK(cudaMemcpy(d_h.p, h.data(), B, cudaMemcpyHostToDevice));

    const double gg = 9.80;                   /* SW2D-EFDC.cu:3977 */
    const double dt = c->dt, dt2 = 2.00 * dt; /* SW2D-EFDC.cu:3976 */
    const double dx = c->cellsize, dy = c->cellsize;
    std::vector<double> rain(c->rain, c->rain + c->nrain);
    rain.resize(c->nrain + 2, 0.0);
    const int nst = c->nst;
    std::vector<double*> qq_rows(c->nqq + 2);
    std::vector<double> qq_store((size_t)(c->nqq + 2) * (nst > 0 ? nst : 1), 0.0);
    for (int j = 0; j < c->nqq + 2; j++) {
        qq_rows[j] = &qq_store[(size_t)j * (nst > 0 ? nst : 1)];
        if (j < c->nqq)
            for (int i = 0; i < nst; i++) qq_rows[j][i] = c->qq[(size_t)j * nst + i];
    }
    std::vector<double> brx(c->brx, c->brx + nst), bry(c->bry, c->bry + nst);

    /* SW2D-EFDC.cu:4763-4766 */
    init_inf<<<numBlocks, threadsPerBlock>>>(rows, cols, d_ho.p, d_h.p, d_inf.p, d_baseo.p, N, c->nodata);
    RCK(cudaDeviceSynchronize());
    initiald<<<numBlocks, threadsPerBlock>>>(rows, cols, d_h.p, d_infx.p, d_infy.p, d_inf.p, d_hm.p, d_hn.p,
                                             d_baseo.p, N, c->nodata);
    RCK(cudaDeviceSynchronize());

    double time = c->time0;
    int mstep = 0;
    long long iters = 0;
    auto wall0 = std::chrono::steady_clock::now();
    while (time + dt <= c->timmax) { /* SW2D-EFDC.cu:4798 */
        if (iters == c->warm_iters) {
            RCK(cudaDeviceSynchronize());
            wall0 = std::chrono::steady_clock::now();
        }
        flux<<<numBlocks, threadsPerBlock>>>(d_th.p, gg, c->manning, d_inf.p, d_h.p, d_infx.p, d_infy.p,
                                             d_baseo.p, d_um.p, d_hm.p, d_uu1.p, d_umo.p, d_vv1.p, d_vva.p,
                                             d_vn.p, d_hn.p, d_vno.p, d_uua.p, d_ho.p, N, cols, rows, dx, dy,
                                             dt2);
        RCK(cudaDeviceSynchronize());
        stream_flow(cols, rows, c->xcoor_c, c->ycoor_c, time, c->dtrain, rain.data(), qq_rows.data(),
                    ql.data(), c->dtoq, brx.data(), bry.data(), dx, dy, nst, &rr);
        RCK(cudaMemcpy(d_ql.p, ql.data(), (size_t)N * sizeof(double), cudaMemcpyHostToDevice));
        RCK(cudaMemcpy(d_rr.p, &rr, sizeof(double), cudaMemcpyHostToDevice));
        continuity<<<numBlocks, threadsPerBlock>>>(dt2, cols, rows, dx, dy, d_rr.p, d_Ev.p, d_ql.p, d_h.p,
                                                   d_ho.p, d_um.p, d_vn.p, c->frac_int, c->frac_inf,
                                                   c->frac_lwl, c->ev_wl_min, d_inf.p, N);
        RCK(cudaDeviceSynchronize());
        treat_error<<<numBlocks, threadsPerBlock>>>(cols, rows, d_th.p, d_inf.p, d_um.p, d_vn.p, d_h.p, N);
        RCK(cudaDeviceSynchronize());
        time = time + dt;
        mstep = mstep + 1;
        stream_flow(cols, rows, c->xcoor_c, c->ycoor_c, time, c->dtrain, rain.data(), qq_rows.data(),
                    ql.data(), c->dtoq, brx.data(), bry.data(), dx, dy, nst, &rr);
        RCK(cudaMemcpy(d_ql.p, ql.data(), (size_t)N * sizeof(double), cudaMemcpyHostToDevice));
        RCK(cudaMemcpy(d_rr.p, &rr, sizeof(double), cudaMemcpyHostToDevice));
        continuity<<<numBlocks, threadsPerBlock>>>(dt2, cols, rows, dx, dy, d_rr.p, d_Ev.p, d_ql.p, d_h.p,
                                                   d_ho.p, d_um.p, d_vn.p, c->frac_int, c->frac_inf,
                                                   c->frac_lwl, c->ev_wl_min, d_inf.p, N);
        RCK(cudaDeviceSynchronize());
        hm_hn<<<numBlocks, threadsPerBlock>>>(d_hm.p, d_hn.p, d_h.p, N, cols, rows);
        RCK(cudaDeviceSynchronize());
        uu1_vv1<<<numBlocks, threadsPerBlock>>>(d_th.p, d_hm.p, d_hn.p, d_uu1.p, d_um.p, d_vv1.p, d_vn.p, N, cols,
                                                rows);
        RCK(cudaDeviceSynchronize());
        uu_vv<<<numBlocks, threadsPerBlock>>>(d_th.p, d_h.p, d_uu1.p, d_vv1.p, d_uu.p, d_vv.p, N, cols);
        RCK(cudaDeviceSynchronize());
        uua_vva<<<numBlocks, threadsPerBlock>>>(d_uu1.p, d_vv1.p, d_uua.p, d_vva.p, N, cols, rows);
        RCK(cudaDeviceSynchronize());
        forward<<<numBlocks, threadsPerBlock>>>(cols, rows, d_umo.p, d_um.p, d_vno.p, d_vn.p, d_ho.p, d_h.p, N);
        RCK(cudaDeviceSynchronize());
        time = time + dt;
        mstep = mstep + 1;
        iters++;
    }
    RCK(cudaDeviceSynchronize());
    o->loop_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    RCK(cudaGetLastError());
    double* outs[7] = {o->h, o->um, o->vn, o->uu, o->vv, o->uua, o->vva};
    double* srcs[7] = {d_h.p, d_um.p, d_vn.p, d_uu.p, d_vv.p, d_uua.p, d_vva.p};
    for (int k = 0; k < 7; k++)
        if (outs[k]) RCK(cudaMemcpy(outs[k], srcs[k], (size_t)N * sizeof(double), cudaMemcpyDeviceToHost));
    o->iters = iters;
    o->time = time;
    o->water_cells = 0;
    o->nqs = 0;
    o->nsamples = 0;
    return 0;
}

} /* extern "C" */
