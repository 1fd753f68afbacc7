/* Host driver of the SW2D step: the C ABI declared in include/sw2d.h.
 *
 * Replaces the reference's host side of the hot path (SW2D-EFDC.cu:4618-4878):
 * instead of nine launches, nine device-wide syncs and two N-double
 * host-to-device copies of the source field per iteration, the forcing of
 * every iteration is prepared on the device by the previous one, and
 * iterations are replayed from a captured CUDA graph with no host round trip
 * until the loop condition is checked at the end of a chunk.
 */
#include "sw2d.h"
#include "sw2d_engine.h"
#include "sw2d_test.h"
#include "sw2d_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <memory>
#include <thread>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace sw2d;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CK(call)                                                                           \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess) {                                                           \
            return fail(e_ == cudaErrorMemoryAllocation ? SW2D_ERR_NOMEM : SW2D_ERR_CUDA,  \
                        std::string(#call) + ": " + cudaGetErrorString(e_));               \
        }                                                                                  \
    } while (0)

constexpr int kChunk = 32; /* iterations per captured graph (even) */

} // namespace

namespace sw2d {
/* sets the message sw2d_last_error returns (for entry points in other units) */
void set_error_message(const char* msg) { g_err = msg; }
} // namespace sw2d

struct sw2d_handle {
    sw2d_config cfg;
    int R = 0, C = 0, P = 0, NR = 0;
    size_t ncell = 0; /* padded cells */
    cudaStream_t stream = nullptr;
    /* device buffers */
    double* z = nullptr;
    uint8_t* flags = nullptr;
    double* h[2] = {nullptr, nullptr};
    double* qx[2] = {nullptr, nullptr};
    double* qy[2] = {nullptr, nullptr};
    double* uu1 = nullptr;
    double* vv1 = nullptr;
    uint8_t* mcls = nullptr;
    double* mtab = nullptr;
    double* gnn = nullptr; /* friction coefficient per class pair */
    int ncls = 0;
    float* rainw = nullptr;
    int* src_idx = nullptr;
    double* rain = nullptr;
    double* evap = nullptr;
    double* srcq = nullptr;
    double* partials = nullptr;
    double* partials_f = nullptr;
    double* outlet = nullptr;
    DevClock* clk = nullptr;
    double* scratch = nullptr; /* 4 * rows * cols doubles, lazily */
    /* host mirrors */
    std::vector<uint8_t> host_flags;
    std::vector<float> host_rainw;
    mutable double active_weight = 0.0; /* sum over active cells of the rain weight */
    mutable bool aw_dirty = false;      /* recomputed when the next launch's parameters are built */
    bool have_dem = false, have_depth = false;
    int nrain = 0, nevap = 0, nsrc = 0, nq = 0, outlet_cap = 0;
    double dtrain = 3600.0, dtoq = 3600.0;
    /* coupling */
    int nfaces = 0, lagged = 1;
    std::vector<int> f_side, f_i, f_j, f_cell;
    void* pin = nullptr;        /* pinned staging of large device-to-host copies */
    size_t pin_bytes = 0;
    int* d_face = nullptr;      /* nfaces * 2: padded cell index, side */
    double* d_face_vel = nullptr;
    double* d_face_q = nullptr;
    /* graph */
    cudaGraphExec_t graph = nullptr;
    bool graph_dirty = true;
    /* timing */
    cudaEvent_t ev_a = nullptr, ev_b = nullptr;
    cudaEvent_t kev[8] = {};
    bool profiling = false;
    double last_ms_per_iter = 0.0;
    std::vector<double> kernel_ms;
    long long prof_iters = 0;
    /* FP32 precision form: a one-scenario engine built from host copies of the inputs */
    std::unique_ptr<sw2d::Engine32> eng;
    int eng_idx = -1;
    std::vector<double> in_dem, in_depth, in_mtab, in_rain, in_evap, in_srcq;
    std::vector<uint8_t> in_mcls;
    std::vector<float> in_rainw;
    std::vector<int> in_srcc;
    int in_nq = 0;
    double in_dtoq = 3600.0;
    bool fp32() const { return cfg.precision == SW2D_FP32; }

    StepParams params() const {
        StepParams p{};
        p.R = R;
        p.C = C;
        p.P = P;
        p.outflow_south = cfg.outflow == SW2D_OUTFLOW_SOUTH;
        p.dt_mode = cfg.dt_mode;
        p.series_mode = cfg.series_mode;
        p.nsrc = nsrc;
        p.nrain = nrain;
        p.nevap = nevap;
        p.nq = nq;
        p.nblocks_cells = ((C + SW2D_BX - 1) / SW2D_BX) * ((R + SW2D_BY - 1) / SW2D_BY);
        p.nblocks_faces = ((C + 1 + SW2D_BX - 1) / SW2D_BX) * ((R + 1 + SW2D_BY - 1) / SW2D_BY);
        p.outlet_cap = outlet_cap;
        p.pct_lake = 1.00 - cfg.frac_lwl;                  /* SW2D-EFDC.cu:627 */
        p.pct_land = 1.00 - (cfg.frac_int + cfg.frac_inf); /* SW2D-EFDC.cu:631 */
        p.ledger_cells = (p.pct_lake != p.pct_land) || (nevap > 0);
        if (aw_dirty) update_active_weight();
        p.rain_static = active_weight * p.pct_land;
        p.dx = cfg.dx;
        p.dy = cfg.dy;
        p.th = cfg.th;
        p.g = cfg.g;
        p.manning = cfg.manning;
        p.ev_wl_min = cfg.ev_wl_min;
        p.dtrain = dtrain;
        p.dtoq = dtoq;
        p.dt_fixed = cfg.dt;
        p.cfl = cfg.cfl;
        p.dt_max = cfg.dt_max;
        p.rdx = 1.0 / cfg.dx;
        p.rdy = 1.0 / cfg.dy;
        p.rsum = p.rdx + p.rdy;
        p.area = cfg.dx * cfg.dy;
        p.flags = flags;
        p.z = z;
        p.mcls = mcls;
        p.mtab = mtab;
        p.gnn = gnn;
        p.ncls = ncls;
        p.gnn_uni = cfg.g * cfg.manning * cfg.manning; /* the reference's gg*rn*rn (SW2D-EFDC.cu:193) */
        auto pow2_exp = [](double d) {
            int k;
            const double m = std::frexp(d, &k); /* d = m 2^k, m in [0.5, 1) */
            return (m == 0.5 && k >= 1 && k <= 31) ? k - 1 : -1;
        };
        p.kdx = pow2_exp(cfg.dx);
        p.kdy = pow2_exp(cfg.dy);
        p.rainw = rainw;
        p.src_idx = src_idx;
        p.rain = rain;
        p.evap = evap;
        p.srcq = srcq;
        for (int k = 0; k < 2; k++) {
            p.h[k] = h[k];
            p.qx[k] = qx[k];
            p.qy[k] = qy[k];
        }
        p.uu1 = uu1;
        p.vv1 = vv1;
        p.partials = partials;
        p.partials_f = partials_f;
        p.outlet = outlet;
        p.clk = clk;
        return p;
    }

    size_t pad_index(int r, int c) const { return (size_t)(r + SW2D_HALO) * P + (c + SW2D_HALO); }

    void update_active_weight() const {
        double s = 0.0;
        for (int r = 0; r < R; r++)
            for (int c = 0; c < C; c++)
                if (host_flags[pad_index(r, c)] & SW2D_F_ACTIVE)
                    s += host_rainw.empty() ? 1.0 : (double)host_rainw[(size_t)r * C + c];
        active_weight = s;
        aw_dirty = false;
    }
};

namespace {

template <typename T>
int dalloc(T** p, size_t n) {
    CK(cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T)));
    CK(cudaMemset(*p, 0, std::max<size_t>(n, 1) * sizeof(T)));
    CK(cudaDeviceSynchronize());
    return SW2D_OK;
}

/* host -> device copy ordered on the handle's stream */
int put(sw2d_handle* h, void* dst, const void* src, size_t bytes);
int zero(sw2d_handle* h, void* dst, size_t bytes);

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

/* Large device-to-host copies go through a pinned staging buffer and a
 * multithreaded host copy: a copy straight into pageable memory runs at a
 * few GB/s (the driver bounces it through its own pinned chunks, one at a
 * time, faulting the destination's fresh pages in as it goes), while a copy
 * into pinned memory runs at the host link's rate. */
constexpr size_t kStageMin = (size_t)4 << 20;

int stage_reserve(sw2d_handle* h, size_t bytes) {
    if (h->pin_bytes >= bytes) return SW2D_OK;
    if (h->pin) cudaFreeHost(h->pin);
    h->pin = nullptr;
    h->pin_bytes = 0;
    CK(cudaMallocHost(&h->pin, bytes));
    h->pin_bytes = bytes;
    return SW2D_OK;
}

/* f(first, last) over [0, n) split across up to 16 host threads */
template <typename F>
void parallel_ranges(size_t n, F f) {
    const size_t nt = std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency(), n / 8 + 1}));
    if (nt == 1) {
        f((size_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    const size_t per = (n + nt - 1) / nt;
    for (size_t t = 0; t < nt; t++) {
        const size_t a = t * per, b = std::min(n, a + per);
        if (a < b) th.emplace_back([=] { f(a, b); });
    }
    for (auto& x : th) x.join();
}

int d2h(sw2d_handle* h, void* dst, const void* src, size_t bytes) {
    if (bytes < kStageMin) {
        CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return SW2D_OK;
    }
    int rc = stage_reserve(h, bytes);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->pin, src, bytes, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const char* s = static_cast<const char*>(h->pin);
    char* d = static_cast<char*>(dst);
    const size_t chunk = (size_t)1 << 20;
    parallel_ranges((bytes + chunk - 1) / chunk, [&](size_t a, size_t b) {
        for (size_t k = a; k < b; k++) std::memcpy(d + k * chunk, s + k * chunk, std::min(chunk, bytes - k * chunk));
    });
    return SW2D_OK;
}

/* Copy a rows x cols host raster into the interior of a padded device field
 * (large rasters: rows laid out with the field's pitch in the pinned staging
 * buffer by host threads, then one copy). */
template <typename T>
int upload_interior(sw2d_handle* h, T* dst, const T* src, int rows, int cols) {
    const size_t rowb = (size_t)h->P * sizeof(T);
    if ((size_t)rows * cols * sizeof(T) < kStageMin) {
        CK(cudaMemcpy2DAsync(dst + h->pad_index(0, 0), rowb, src, (size_t)cols * sizeof(T),
                             (size_t)cols * sizeof(T), rows, cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return SW2D_OK;
    }
    int rc = stage_reserve(h, (size_t)rows * rowb);
    if (rc) return rc;
    T* s = static_cast<T*>(h->pin);
    const size_t P = (size_t)h->P;
    parallel_ranges((size_t)rows, [&](size_t a, size_t b) {
        for (size_t r = a; r < b; r++) std::memcpy(s + r * P, src + r * cols, (size_t)cols * sizeof(T));
    });
    /* the staged rows' pitch columns outside the interior are not copied */
    CK(cudaMemcpy2DAsync(dst + h->pad_index(0, 0), rowb, s, rowb, (size_t)cols * sizeof(T), rows,
                         cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

template <typename T>
int download_block(sw2d_handle* h, T* dst, const T* src_padded, int r0, int c0, int rows, int cols) {
    const size_t rowb = (size_t)h->P * sizeof(T);
    if ((size_t)rows * cols * sizeof(T) < kStageMin) {
        CK(cudaMemcpy2DAsync(dst, (size_t)cols * sizeof(T), src_padded + h->pad_index(r0, c0), rowb,
                             (size_t)cols * sizeof(T), rows, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return SW2D_OK;
    }
    /* whole padded rows into the staging buffer, then the interior columns out */
    int rc = stage_reserve(h, (size_t)rows * rowb);
    if (rc) return rc;
    CK(cudaMemcpyAsync(h->pin, src_padded + (size_t)(r0 + SW2D_HALO) * h->P, (size_t)rows * rowb,
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const T* s = static_cast<const T*>(h->pin) + (c0 + SW2D_HALO);
    const size_t P = (size_t)h->P;
    parallel_ranges((size_t)rows, [&](size_t a, size_t b) {
        for (size_t r = a; r < b; r++) std::memcpy(dst + r * cols, s + r * P, (size_t)cols * sizeof(T));
    });
    return SW2D_OK;
}

int put(sw2d_handle* h, void* dst, const void* src, size_t bytes) {
    if (bytes >= kStageMin && stage_reserve(h, bytes) == SW2D_OK) {
        const char* sp = static_cast<const char*>(src);
        char* d = static_cast<char*>(h->pin);
        const size_t chunk = (size_t)1 << 20;
        parallel_ranges((bytes + chunk - 1) / chunk, [&](size_t a, size_t b) {
            for (size_t k = a; k < b; k++)
                std::memcpy(d + k * chunk, sp + k * chunk, std::min(chunk, bytes - k * chunk));
        });
        src = h->pin;
    }
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

int zero(sw2d_handle* h, void* dst, size_t bytes) {
    CK(cudaMemsetAsync(dst, 0, bytes, h->stream));
    return SW2D_OK;
}

int sync_check(sw2d_handle* h) {
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    return SW2D_OK;
}

int set_device(sw2d_handle* h) {
    CK(cudaSetDevice(h->cfg.device));
    return SW2D_OK;
}

int read_clock(sw2d_handle* h, DevClock* out) {
    CK(cudaMemcpyAsync(out, h->clk, sizeof(DevClock), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return SW2D_OK;
}

/* full = 0: recompute the next iteration's slot (after t_end or forcing
 * changed); 1: volume of the current state only, the clock untouched;
 * 2: initial state (volume origin, CFL speed, first slot). */
int prime(sw2d_handle* h, int full) {
    StepParams p = h->params();
    fp64_launch_prime(p, 0, full, h->stream);
    return sync_check(h);
}

int build_graph(sw2d_handle* h) {
    if (h->graph && !h->graph_dirty) return SW2D_OK;
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    StepParams p = h->params();
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kChunk; k++) fp64_launch_iteration(p, k & 1, h->stream, nullptr);
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(SW2D_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    h->graph_dirty = false;
    return SW2D_OK;
}

/* Launch n (even) iterations starting from buffer 0. */
int launch_iterations(sw2d_handle* h, long long n) {
    if (n <= 0) return SW2D_OK;
    if (h->profiling) {
        StepParams p = h->params();
        const int nk = fp64_kernels_per_iteration();
        for (long long k = 0; k < n; k++) {
            fp64_launch_iteration(p, (int)(k & 1), h->stream, h->kev);
            CK(cudaEventSynchronize(h->kev[nk]));
            for (int j = 0; j < nk; j++) {
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, h->kev[j], h->kev[j + 1]));
                h->kernel_ms[j] += ms;
            }
            h->prof_iters++;
        }
        return sync_check(h);
    }
    int rc = build_graph(h);
    if (rc) return rc;
    long long full = n / kChunk, rem = n % kChunk;
    for (long long k = 0; k < full; k++) CK(cudaGraphLaunch(h->graph, h->stream));
    StepParams p = h->params();
    for (long long k = 0; k < rem; k++) fp64_launch_iteration(p, (int)(k & 1), h->stream, nullptr);
    CK(cudaGetLastError());
    return SW2D_OK;
}

int fp32_rebuild(sw2d_handle* h) {
    if (h->eng_idx >= 0) {
        h->eng->remove(h->eng_idx);
        h->eng_idx = -1;
    }
    sw2d::ScenarioInput in;
    const sw2d_config& c = h->cfg;
    in.rows = c.rows;
    in.cols = c.cols;
    in.dx = c.dx;
    in.dy = c.dy;
    in.nodata = c.nodata;
    in.th = c.th;
    in.g = c.g;
    in.manning = c.manning;
    in.dt_mode = c.dt_mode;
    in.series_mode = c.series_mode;
    in.outflow_south = c.outflow == SW2D_OUTFLOW_SOUTH;
    in.dt = c.dt;
    in.cfl = c.cfl;
    in.dt_max = c.dt_max;
    in.t0 = c.t0;
    in.t_end = c.t0;
    in.frac_int = c.frac_int;
    in.frac_inf = c.frac_inf;
    in.frac_lwl = c.frac_lwl;
    in.ev_wl_min = c.ev_wl_min;
    in.dem = h->in_dem.data();
    in.depth = h->in_depth.data();
    if (!h->in_mcls.empty()) {
        in.mclass = h->in_mcls.data();
        in.mtable = h->in_mtab.data();
        in.ntable = (int)h->in_mtab.size();
    }
    in.rain = h->in_rain.data();
    in.nrain = (int)h->in_rain.size();
    in.dtrain = h->dtrain;
    if (!h->in_rainw.empty()) in.rain_weight = h->in_rainw.data();
    if (!h->in_evap.empty()) {
        in.evap = h->in_evap.data();
        in.nevap = (int)h->in_evap.size();
    }
    if (!h->in_srcc.empty()) {
        in.nsrc = (int)h->in_srcc.size();
        in.src_cells = h->in_srcc.data();
        in.src_q = h->in_srcq.data();
        in.nq = h->in_nq;
        in.dtoq = h->in_dtoq;
    }
    in.outlet_cap = h->outlet_cap;
    std::string err;
    int rc = h->eng->add(in, 0, &err, &h->eng_idx);
    if (rc) return fail(rc, err);
    return SW2D_OK;
}

int check_ready(sw2d_handle* h) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (!h->have_dem || !h->have_depth) return fail(SW2D_ERR_STATE, "set_dem and set_depth must be called first");
    return set_device(h);
}

int run_until_fp32(sw2d_handle* h, double t_end, long long max_iters, int64_t* done_out) {
    std::string err;
    int rc = h->eng->set_t_end(h->eng_idx, t_end, &err);
    if (rc) return fail(rc, err);
    sw2d::Clock32 c0, c;
    if ((rc = h->eng->get_clock(h->eng_idx, &c0, &err))) return fail(rc, err);
    double ms = 0;
    if (max_iters >= 0) {
        if ((rc = h->eng->run(max_iters, &err))) return fail(rc, err);
        ms = h->eng->last_ms();
    } else {
        for (;;) {
            if ((rc = h->eng->run(64, &err))) return fail(rc, err);
            ms += h->eng->last_ms();
            if ((rc = h->eng->get_clock(h->eng_idx, &c, &err))) return fail(rc, err);
            if (c.done || !c.slot.active) break;
            if (c.status & 7) break;
        }
    }
    if ((rc = h->eng->get_clock(h->eng_idx, &c, &err))) return fail(rc, err);
    const long long done = c.iters - c0.iters;
    h->last_ms_per_iter = done > 0 ? ms / (double)done : 0.0;
    if (done_out) *done_out = done;
    if (c.status & 4) return fail(SW2D_ERR_CUDA, "FP32 tile staging buffer misaligned (tiles skipped)");
    if (c.status & 2) return fail(SW2D_ERR_TIMEOUT, "a tile's staged load did not arrive in time");
    if (c.status & 1) return fail(SW2D_ERR_NUMERIC, "non-finite state");
    return SW2D_OK;
}

int run_until(sw2d_handle* h, double t_end, long long max_iters, int64_t* done_out) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->fp32()) return run_until_fp32(h, t_end, max_iters, done_out);
    if ((rc = put(h, &h->clk->t_end, &t_end, sizeof(double)))) return rc;
    if ((rc = prime(h, 0))) return rc;
    DevClock c0;
    if ((rc = read_clock(h, &c0))) return rc;
    const long long it0 = c0.iters;
    CK(cudaEventRecord(h->ev_a, h->stream));
    long long launched = 0;
    if (h->cfg.dt_mode == SW2D_DT_FIXED) {
        /* the reference's loop condition, replayed on the host to size the launch */
        double t = c0.t, dt = h->cfg.dt;
        long long n = 0;
        while (t + dt <= t_end && (max_iters < 0 || n < max_iters)) {
            t = (t + dt) + dt;
            n++;
        }
        long long ne = n + (n & 1);
        if (max_iters >= 0 && (n & 1)) {
            /* an odd bounded count: the extra iteration must not advance */
            double te = t;
            if ((rc = put(h, &h->clk->t_end, &te, sizeof(double)))) return rc;
            if ((rc = prime(h, 0))) return rc;
        }
        if ((rc = launch_iterations(h, ne))) return rc;
        launched = ne;
    } else if (max_iters >= 0) {
        /* a bounded CFL run: an odd count launches one iteration more, which
         * the device's iteration limit leaves inactive (a state copy), so the
         * state ends in buffer 0 as the captured pairs need */
        const long long ne = max_iters + (max_iters & 1);
        if (max_iters & 1) {
            const long long lim = it0 + max_iters;
            if ((rc = put(h, &h->clk->iter_end, &lim, sizeof lim))) return rc;
            if ((rc = prime(h, 0))) return rc;
        }
        rc = launch_iterations(h, ne);
        if (max_iters & 1) {
            const long long none = LLONG_MAX;
            const int rc2 = put(h, &h->clk->iter_end, &none, sizeof none);
            if (!rc) rc = rc2;
        }
        if (rc) return rc;
        launched = ne;
    } else {
        for (;;) {
            if ((rc = launch_iterations(h, kChunk))) return rc;
            launched += kChunk;
            DevClock c;
            if ((rc = read_clock(h, &c))) return rc;
            if (!c.slot[0].active) break;
            if (c.status & 1) return fail(SW2D_ERR_NUMERIC, "non-finite depth");
        }
    }
    CK(cudaEventRecord(h->ev_b, h->stream));
    CK(cudaEventSynchronize(h->ev_b));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, h->ev_a, h->ev_b));
    DevClock c1;
    if ((rc = read_clock(h, &c1))) return rc;
    long long done = c1.iters - it0;
    h->last_ms_per_iter = done > 0 ? ms / (double)done : 0.0;
    if (done_out) *done_out = done;
    if (c1.status & 1) return fail(SW2D_ERR_NUMERIC, "non-finite depth");
    (void)launched;
    /* restore the open-ended t_end in the clock slot for later queries */
    return SW2D_OK;
}

} // namespace

extern "C" {

int sw2d_abi_version(void) { return SW2D_ABI_VERSION; }

const char* sw2d_last_error(void) { return g_err.c_str(); }

const char* sw2d_status_string(int s) {
    switch (s) {
    case SW2D_OK: return "ok";
    case SW2D_ERR_INVALID: return "invalid argument";
    case SW2D_ERR_CUDA: return "CUDA error";
    case SW2D_ERR_NOMEM: return "out of memory";
    case SW2D_ERR_STATE: return "invalid state";
    case SW2D_ERR_BUDGET: return "HBM budget exceeded";
    case SW2D_ERR_NUMERIC: return "non-finite state";
    case SW2D_ERR_NODEVICE: return "no sm_103 device";
    case SW2D_ERR_TIMEOUT: return "timeout";
    case SW2D_ERR_NOT_FOUND: return "not found";
    case SW2D_ERR_IO: return "file error";
    default: return "unknown";
    }
}

int sw2d_config_default(sw2d_config* c) {
    if (!c) return fail(SW2D_ERR_INVALID, "null config");
    std::memset(c, 0, sizeof(*c));
    c->precision = SW2D_FP64;
    c->dt_mode = SW2D_DT_FIXED;
    c->series_mode = SW2D_SERIES_REFERENCE;
    c->outflow = SW2D_OUTFLOW_NONE;
    c->dx = c->dy = 10.0;
    c->nodata = -9999.0;
    c->th = 1.0e-4;
    c->g = 9.80;
    c->manning = 0.03;
    c->dt = 0.04;
    c->cfl = 0.7;
    c->dt_max = 1.0;
    c->ev_wl_min = 0.05;
    return SW2D_OK;
}

int sw2d_create(const sw2d_config* cfg, sw2d_handle** out) {
    if (!cfg || !out) return fail(SW2D_ERR_INVALID, "null argument");
    *out = nullptr;
    if (cfg->rows < 2 || cfg->cols < 2) return fail(SW2D_ERR_INVALID, "rows and cols must be >= 2");
    if ((long long)cfg->rows * cfg->cols > (1LL << 31) / 2) return fail(SW2D_ERR_INVALID, "raster too large");
    if (!(cfg->dx > 0) || !(cfg->dy > 0)) return fail(SW2D_ERR_INVALID, "dx, dy must be > 0");
    if (!(cfg->th > 0)) return fail(SW2D_ERR_INVALID, "th must be > 0");
    if (cfg->precision != SW2D_FP64 && cfg->precision != SW2D_FP32) return fail(SW2D_ERR_INVALID, "precision");
    if (cfg->dt_mode == SW2D_DT_FIXED && !(cfg->dt > 0)) return fail(SW2D_ERR_INVALID, "dt must be > 0");
    if (cfg->dt_mode == SW2D_DT_CFL && (!(cfg->cfl > 0) || !(cfg->dt_max > 0)))
        return fail(SW2D_ERR_INVALID, "cfl and dt_max must be > 0");
    if (cfg->dt_mode != SW2D_DT_FIXED && cfg->dt_mode != SW2D_DT_CFL) return fail(SW2D_ERR_INVALID, "dt_mode");
    if (cfg->series_mode < 0 || cfg->series_mode > 2) return fail(SW2D_ERR_INVALID, "series_mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= cfg->device || cfg->device < 0)
        return fail(SW2D_ERR_NODEVICE, "no CUDA device");
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, cfg->device));
    if (prop.major != 10 || prop.minor != 3)
        return fail(SW2D_ERR_NODEVICE, "this library is built for sm_103a (GB300) only");
    sw2d_handle* h = new sw2d_handle();
    h->cfg = *cfg;
    if (cfg->precision == SW2D_FP32) {
        h->R = cfg->rows;
        h->C = cfg->cols;
        const size_t need = sw2d::Engine32::scenario_bytes(cfg->rows, cfg->cols, false, 0);
        if (cfg->hbm_budget_bytes > 0 && (double)need > cfg->hbm_budget_bytes) {
            delete h;
            return fail(SW2D_ERR_BUDGET, "model does not fit the HBM budget");
        }
        h->eng.reset(new sw2d::Engine32(cfg->device));
        std::string err;
        int rc0 = h->eng->init(&err);
        if (rc0) {
            delete h;
            return fail(rc0, err);
        }
        h->in_rain.assign(1, 0.0);
        *out = h;
        return SW2D_OK;
    }
    h->R = cfg->rows;
    h->C = cfg->cols;
    h->P = ((cfg->cols + 2 * SW2D_HALO + 31) / 32) * 32;
    h->NR = cfg->rows + 2 * SW2D_HALO;
    h->ncell = (size_t)h->NR * h->P;
    const size_t need = h->ncell * (8 * 7 + 2) + 4096;
    if (cfg->hbm_budget_bytes > 0 && (double)need > cfg->hbm_budget_bytes) {
        delete h;
        return fail(SW2D_ERR_BUDGET, "model does not fit the HBM budget");
    }
    int rc;
#define TRY(x)                   \
    if ((rc = (x)) != SW2D_OK) { \
        sw2d_destroy(h);         \
        return rc;               \
    }
    TRY(set_device(h));
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(SW2D_ERR_CUDA, "stream");
    }
    TRY(dalloc(&h->z, h->ncell));
    TRY(dalloc(&h->flags, h->ncell));
    for (int k = 0; k < 2; k++) {
        TRY(dalloc(&h->h[k], h->ncell));
        TRY(dalloc(&h->qx[k], h->ncell));
        TRY(dalloc(&h->qy[k], h->ncell));
    }
    TRY(dalloc(&h->uu1, h->ncell));
    TRY(dalloc(&h->vv1, h->ncell));
    TRY(dalloc(&h->partials, (size_t)h->params().nblocks_cells * 4 + 8));
    TRY(dalloc(&h->partials_f, (size_t)h->params().nblocks_faces * 2 + 8));
    TRY(dalloc(&h->clk, 1));
    TRY(dalloc(&h->rain, 4));
    TRY(dalloc(&h->srcq, 4));
    h->nrain = 1;
    if (cudaEventCreate(&h->ev_a) != cudaSuccess || cudaEventCreate(&h->ev_b) != cudaSuccess) {
        sw2d_destroy(h);
        return fail(SW2D_ERR_CUDA, "events");
    }
    for (int k = 0; k < 8; k++) cudaEventCreate(&h->kev[k]);
    h->kernel_ms.assign(8, 0.0);
    DevClock c{};
    c.iter_end = LLONG_MAX;
    c.t = cfg->t0;
    c.t_end = cfg->t0;
    if (cudaMemcpy(h->clk, &c, sizeof c, cudaMemcpyHostToDevice) != cudaSuccess) {
        sw2d_destroy(h);
        return fail(SW2D_ERR_CUDA, "clock init");
    }
    h->host_flags.assign(h->ncell, 0);
#undef TRY
    *out = h;
    return SW2D_OK;
}

int sw2d_destroy(sw2d_handle* h) {
    if (!h) return SW2D_OK;
    if (h->fp32()) {
        h->eng.reset();
        if (h->pin) cudaFreeHost(h->pin);
        delete h;
        return SW2D_OK;
    }
    cudaSetDevice(h->cfg.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    dfree(h->z);
    dfree(h->flags);
    for (int k = 0; k < 2; k++) {
        dfree(h->h[k]);
        dfree(h->qx[k]);
        dfree(h->qy[k]);
    }
    dfree(h->uu1);
    dfree(h->vv1);
    dfree(h->mcls);
    dfree(h->mtab);
    dfree(h->gnn);
    dfree(h->rainw);
    dfree(h->src_idx);
    dfree(h->rain);
    dfree(h->evap);
    dfree(h->srcq);
    dfree(h->partials);
    dfree(h->partials_f);
    dfree(h->outlet);
    dfree(h->clk);
    dfree(h->scratch);
    dfree(h->d_face);
    dfree(h->d_face_vel);
    dfree(h->d_face_q);
    if (h->ev_a) cudaEventDestroy(h->ev_a);
    if (h->ev_b) cudaEventDestroy(h->ev_b);
    for (int k = 0; k < 8; k++)
        if (h->kev[k]) cudaEventDestroy(h->kev[k]);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->pin) cudaFreeHost(h->pin);
    delete h;
    return SW2D_OK;
}

int sw2d_set_dem(sw2d_handle* h, const double* zin) {
    if (!h || !zin) return fail(SW2D_ERR_INVALID, "null argument");
    if (h->fp32()) {
        h->in_dem.assign(zin, zin + (size_t)h->R * h->C);
        h->have_dem = true;
        return SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    if ((rc = upload_interior(h, h->z, zin, h->R, h->C))) return rc;
    std::fill(h->host_flags.begin(), h->host_flags.end(), 0);
    parallel_ranges((size_t)h->R, [&](size_t a, size_t b) {
        for (size_t r = a; r < b; r++)
            for (int c = 0; c < h->C; c++) {
                const double v = zin[r * h->C + c];
                h->host_flags[h->pad_index((int)r, c)] = (v != h->cfg.nodata) ? SW2D_F_ACTIVE : 0; /* :37-42 */
            }
    });
    for (int k = 0; k < h->nsrc; k++) {
        /* source flags are re-applied by set_point_sources */
    }
    if ((rc = put(h, h->flags, h->host_flags.data(), h->ncell))) return rc;
    h->aw_dirty = true;
    h->have_dem = true;
    h->graph_dirty = true;
    return SW2D_OK;
}

int sw2d_set_depth(sw2d_handle* h, const double* d) {
    if (!h || !d) return fail(SW2D_ERR_INVALID, "null argument");
    if (!h->have_dem) return fail(SW2D_ERR_STATE, "set_dem first");
    if (h->fp32()) {
        h->in_depth.assign(d, d + (size_t)h->R * h->C);
        h->have_depth = true;
        return fp32_rebuild(h);
    }
    int rc = set_device(h);
    if (rc) return rc;
    std::vector<double> dd(d, d + (size_t)h->R * h->C);
    for (int r = 0; r < h->R; r++)
        for (int c = 0; c < h->C; c++)
            if (!(h->host_flags[h->pad_index(r, c)] & SW2D_F_ACTIVE)) dd[(size_t)r * h->C + c] = 0.0;
    for (int k = 0; k < 2; k++) {
        if ((rc = zero(h, h->h[k], h->ncell * sizeof(double)))) return rc;
        if ((rc = zero(h, h->qx[k], h->ncell * sizeof(double)))) return rc;
        if ((rc = zero(h, h->qy[k], h->ncell * sizeof(double)))) return rc;
    }
    if ((rc = zero(h, h->uu1, h->ncell * sizeof(double)))) return rc;
    if ((rc = zero(h, h->vv1, h->ncell * sizeof(double)))) return rc;
    if ((rc = upload_interior(h, h->h[0], dd.data(), h->R, h->C))) return rc;
    DevClock c{};
    c.iter_end = LLONG_MAX;
    c.t = h->cfg.t0;
    c.t_end = h->cfg.t0;
    if ((rc = put(h, h->clk, &c, sizeof c))) return rc;
    h->have_depth = true;
    return prime(h, 2);
}

int sw2d_set_manning_classes(sw2d_handle* h, const uint8_t* cls, const double* table, int ntable) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (h->fp32()) {
        if (!cls) {
            h->in_mcls.clear();
            h->in_mtab.clear();
        } else {
            if (!table || ntable <= 0 || ntable > 64) return fail(SW2D_ERR_INVALID, "manning table (FP32: <= 64 classes)");
            for (size_t k = 0; k < (size_t)h->R * h->C; k++)
                if (cls[k] >= ntable) return fail(SW2D_ERR_INVALID, "manning class out of table range");
            h->in_mcls.assign(cls, cls + (size_t)h->R * h->C);
            h->in_mtab.assign(table, table + ntable);
        }
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    if (!cls) {
        dfree(h->mcls);
        dfree(h->mtab);
        dfree(h->gnn);
        h->ncls = 0;
        h->graph_dirty = true;
        return SW2D_OK;
    }
    if (!table || ntable <= 0 || ntable > 256) return fail(SW2D_ERR_INVALID, "manning table");
    for (size_t k = 0; k < (size_t)h->R * h->C; k++)
        if (cls[k] >= ntable) return fail(SW2D_ERR_INVALID, "manning class out of table range");
    if (!h->mcls && (rc = dalloc(&h->mcls, h->ncell))) return rc;
    dfree(h->mtab);
    if ((rc = dalloc(&h->mtab, 256))) return rc;
    CK(cudaMemcpy(h->mtab, table, sizeof(double) * ntable, cudaMemcpyHostToDevice));
    /* the friction coefficient (g n_f) n_f of every class pair, n_f the mean
     * of the two cells' n, with the reference's operations in its order
     * (SW2D-EFDC.cu:193, :310); up to 32 classes, else per face */
    dfree(h->gnn);
    h->ncls = 0;
    if (ntable <= 32) {
        std::vector<double> g2((size_t)ntable * ntable);
        for (int a = 0; a < ntable; a++)
            for (int b = 0; b < ntable; b++) {
                const double nf = 0.50 * (table[a] + table[b]);
                g2[(size_t)a * ntable + b] = h->cfg.g * nf * nf;
            }
        if ((rc = dalloc(&h->gnn, g2.size()))) return rc;
        CK(cudaMemcpy(h->gnn, g2.data(), sizeof(double) * g2.size(), cudaMemcpyHostToDevice));
        h->ncls = ntable;
    }
    if ((rc = upload_interior(h, h->mcls, cls, h->R, h->C))) return rc;
    h->graph_dirty = true;
    return SW2D_OK;
}

int sw2d_set_manning_field(sw2d_handle* h, const double* n) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (!n) return sw2d_set_manning_classes(h, nullptr, nullptr, 0);
    const int64_t cells = (int64_t)h->R * h->C;
    std::vector<uint8_t> cls((size_t)cells);
    double table[256];
    int ntable = 0;
    int rc = sw2d_manning_classes_of(cells, n, h->fp32() ? 64 : 256, cls.data(), table, &ntable);
    if (rc) return rc;
    return sw2d_set_manning_classes(h, cls.data(), table, ntable);
}

int sw2d_set_rain_series(sw2d_handle* h, const double* mm, int n, double dtrain) {
    if (!h || (n > 0 && !mm) || n < 0 || !(dtrain > 0)) return fail(SW2D_ERR_INVALID, "rain series");
    if (h->fp32()) {
        h->in_rain.assign(mm, mm + n);
        if (n == 0) h->in_rain.assign(1, 0.0);
        h->dtrain = dtrain;
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    /* nrain entries and the two-entry zero tail the clamped lookup reads */
    std::vector<double> v((size_t)std::max(n, 1) + 2, 0.0);
    for (int k = 0; k < n; k++) v[k] = mm[k];
    dfree(h->rain);
    if ((rc = dalloc(&h->rain, v.size()))) return rc;
    CK(cudaMemcpy(h->rain, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
    h->nrain = std::max(n, 1);
    h->dtrain = dtrain;
    h->graph_dirty = true;
    return h->have_depth ? prime(h, 0) : SW2D_OK;
}

int sw2d_set_rain_field(sw2d_handle* h, const float* w) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (h->fp32()) {
        if (w) h->in_rainw.assign(w, w + (size_t)h->R * h->C);
        else h->in_rainw.clear();
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    if (!w) {
        dfree(h->rainw);
        h->host_rainw.clear();
    } else {
        if (!h->rainw && (rc = dalloc(&h->rainw, h->ncell))) return rc;
        if ((rc = upload_interior(h, h->rainw, w, h->R, h->C))) return rc;
        h->host_rainw.assign(w, w + (size_t)h->R * h->C);
    }
    h->aw_dirty = true;
    h->graph_dirty = true;
    return SW2D_OK;
}

int sw2d_set_evaporation_series(sw2d_handle* h, const double* mm, int n) {
    if (!h || n < 0 || (n > 0 && !mm)) return fail(SW2D_ERR_INVALID, "evaporation series");
    if (h->fp32()) {
        h->in_evap.assign(mm, mm + n);
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    dfree(h->evap);
    h->nevap = 0;
    if (n > 0) {
        std::vector<double> v(n + 2, 0.0);
        for (int k = 0; k < n; k++) v[k] = mm[k];
        if ((rc = dalloc(&h->evap, v.size()))) return rc;
        CK(cudaMemcpy(h->evap, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
        h->nevap = n;
    }
    h->graph_dirty = true;
    return h->have_depth ? prime(h, 0) : SW2D_OK;
}

int sw2d_set_point_sources(sw2d_handle* h, int nsrc, const int* cells, const double* q, int nq, double dtoq) {
    if (!h || nsrc < 0 || nsrc > SW2D_MAX_SRC || (nsrc > 0 && (!cells || !q || nq <= 0 || !(dtoq > 0))))
        return fail(SW2D_ERR_INVALID, "point sources");
    if (!h->have_dem) return fail(SW2D_ERR_STATE, "set_dem first");
    if (h->fp32()) {
        for (int k = 0; k < nsrc; k++)
            if (cells[k] < 0 || cells[k] >= h->R * h->C) return fail(SW2D_ERR_INVALID, "source cell out of range");
        h->in_srcc.assign(cells, cells + nsrc);
        h->in_srcq.assign(q, q + (size_t)nq * nsrc);
        h->in_nq = nsrc > 0 ? nq : 0;
        h->in_dtoq = nsrc > 0 ? dtoq : 3600.0;
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    int rc = set_device(h);
    if (rc) return rc;
    for (size_t i = 0; i < h->ncell; i++) h->host_flags[i] &= (uint8_t)~SW2D_F_SOURCE;
    std::vector<int> idx(std::max(nsrc, 1), -1);
    for (int k = 0; k < nsrc; k++) {
        if (cells[k] < 0 || cells[k] >= h->R * h->C) return fail(SW2D_ERR_INVALID, "source cell out of range");
        int r = cells[k] / h->C, c = cells[k] % h->C;
        idx[k] = (int)h->pad_index(r, c);
        h->host_flags[idx[k]] |= SW2D_F_SOURCE;
    }
    /* the reference writes each source into ql[cell] in order, so a later
     * source on the same cell wins (stream_flow :541-544) */
    for (int k = 0; k < nsrc; k++)
        for (int j = k + 1; j < nsrc; j++)
            if (idx[j] == idx[k]) idx[k] = -2;
    if ((rc = put(h, h->flags, h->host_flags.data(), h->ncell))) return rc;
    dfree(h->src_idx);
    dfree(h->srcq);
    if ((rc = dalloc(&h->src_idx, idx.size()))) return rc;
    CK(cudaMemcpy(h->src_idx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
    std::vector<double> v((size_t)(nq + 2) * std::max(nsrc, 1), 0.0);
    for (size_t k = 0; k < (size_t)nq * nsrc; k++) v[k] = q[k];
    if ((rc = dalloc(&h->srcq, v.size()))) return rc;
    CK(cudaMemcpy(h->srcq, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
    h->nsrc = nsrc;
    h->nq = nq;
    h->dtoq = nsrc > 0 ? dtoq : 3600.0;
    h->graph_dirty = true;
    return h->have_depth ? prime(h, 0) : SW2D_OK;
}

int sw2d_advance(sw2d_handle* h, double t_end, int64_t* iterations_out) {
    sw2d::NvtxRange r("sw2d_advance");
    return run_until(h, t_end, -1, iterations_out);
}

int sw2d_step(sw2d_handle* h, int n, double t_end) {
    sw2d::NvtxRange r("sw2d_step");
    if (n < 0) return fail(SW2D_ERR_INVALID, "n < 0");
    int64_t done = 0;
    return run_until(h, t_end, n, &done);
}

int sw2d_get_time(sw2d_handle* h, double* t, int64_t* iters) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    int rc = set_device(h);
    if (rc) return rc;
    if (h->fp32()) {
        if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
        sw2d::Clock32 c;
        std::string err;
        if ((rc = h->eng->get_clock(h->eng_idx, &c, &err))) return fail(rc, err);
        if (t) *t = c.t;
        if (iters) *iters = c.iters;
        return SW2D_OK;
    }
    DevClock c;
    if ((rc = read_clock(h, &c))) return rc;
    if (t) *t = c.t;
    if (iters) *iters = c.iters;
    return SW2D_OK;
}

int sw2d_get_state(sw2d_handle* h, double* depth, double* qx, double* qy) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->fp32()) {
        std::string err;
        if ((rc = h->eng->get_state(h->eng_idx, depth, qx, qy, &err))) return fail(rc, err);
        return SW2D_OK;
    }
    if (depth && (rc = download_block(h, depth, h->h[0], 0, 0, h->R, h->C))) return rc;
    if (qx && (rc = download_block(h, qx, h->qx[0], 0, 0, h->R + 1, h->C))) return rc;
    if (qy && (rc = download_block(h, qy, h->qy[0], 0, 0, h->R, h->C + 1))) return rc;
    return SW2D_OK;
}

/* FP32 handles: the reference's uu1_vv1 / uu_vv / uua_vva formulas
 * (SW2D-EFDC.cu:404-522) applied to the downloaded state, for output. */
static int velocities_fp32(sw2d_handle* h, double* uu, double* vv, double* uua, double* vva) {
    const int R = h->R, C = h->C;
    std::vector<double> d((size_t)R * C), qx((size_t)(R + 1) * C), qy((size_t)R * (C + 1));
    std::string err;
    int rc = h->eng->get_state(h->eng_idx, d.data(), qx.data(), qy.data(), &err);
    if (rc) return fail(rc, err);
    const double th = h->cfg.th;
    std::vector<double> u1((size_t)(R + 1) * C, 0.0), v1((size_t)R * (C + 1), 0.0);
    for (int r = 0; r <= R; r++)
        for (int c = 0; c < C; c++) {
            double hm = r == 0 ? d[c] : (r == R ? d[(size_t)(R - 1) * C + c] : 0.5 * (d[(size_t)r * C + c] + d[(size_t)(r - 1) * C + c]));
            double q = qx[(size_t)r * C + c];
            u1[(size_t)r * C + c] = hm >= th ? q / hm : 0.0;
        }
    for (int r = 0; r < R; r++)
        for (int c = 0; c <= C; c++) {
            double hn = c == 0 ? d[(size_t)r * C] : (c == C ? d[(size_t)r * C + C - 1] : 0.5 * (d[(size_t)r * C + c] + d[(size_t)r * C + c - 1]));
            double q = qy[(size_t)r * (C + 1) + c];
            v1[(size_t)r * (C + 1) + c] = hn >= th ? q / hn : 0.0;
        }
    auto U = [&](int r, int c) { return u1[(size_t)r * C + c]; };
    auto V = [&](int r, int c) { return v1[(size_t)r * (C + 1) + c]; };
    for (int r = 0; r < R; r++)
        for (int c = 0; c < C; c++) {
            const size_t k = (size_t)r * C + c;
            const bool wet = d[k] >= th;
            if (uu) uu[k] = wet ? (U(r + 1, c) + U(r, c)) / 2.00 : 0.0;
            if (vv) vv[k] = wet ? (V(r, c + 1) + V(r, c)) / 2.00 : 0.0;
            if (uua) uua[k] = c > 0 ? 0.250 * (U(r, c) + U(r + 1, c) + U(r, c - 1) + U(r + 1, c - 1)) : 0.50 * (U(r, c) + U(r + 1, c));
            if (vva) vva[k] = r > 0 ? 0.250 * (V(r, c) + V(r, c + 1) + V(r - 1, c) + V(r - 1, c + 1)) : 0.50 * (V(r, c) + V(r, c + 1));
        }
    return SW2D_OK;
}

static int velocities(sw2d_handle* h, double* uu, double* vv, double* uua, double* vva) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->fp32()) return velocities_fp32(h, uu, vv, uua, vva);
    const size_t n = (size_t)h->R * h->C;
    if (!h->scratch && (rc = dalloc(&h->scratch, 4 * n))) return rc;
    StepParams p = h->params();
    fp64_launch_cell_velocity(p, 0, uu ? h->scratch : nullptr, vv ? h->scratch + n : nullptr,
                              uua ? h->scratch + 2 * n : nullptr, vva ? h->scratch + 3 * n : nullptr, h->stream);
    if ((rc = sync_check(h))) return rc;
    double* outs[4] = {uu, vv, uua, vva};
    for (int k = 0; k < 4; k++)
        if (outs[k] && (rc = d2h(h, outs[k], h->scratch + k * n, n * sizeof(double)))) return rc;
    return SW2D_OK;
}

int sw2d_get_velocity(sw2d_handle* h, double* uu, double* vv) { return velocities(h, uu, vv, nullptr, nullptr); }

int sw2d_get_face_velocity(sw2d_handle* h, double* uua, double* vva) {
    return velocities(h, nullptr, nullptr, uua, vva);
}

int sw2d_get_ledger(sw2d_handle* h, sw2d_ledger* out) {
    if (!h || !out) return fail(SW2D_ERR_INVALID, "null argument");
    int rc = set_device(h);
    if (rc) return rc;
    if (h->fp32()) {
        if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
        sw2d::Clock32 c;
        std::string err;
        double vol = 0, smax = 0;
        if ((rc = h->eng->get_clock(h->eng_idx, &c, &err))) return fail(rc, err);
        if ((rc = h->eng->get_volume(h->eng_idx, &vol, &smax, &err))) return fail(rc, err);
        out->time = c.t;
        out->iterations = (double)c.iters;
        out->volume = vol;
        out->volume0 = c.volume0;
        out->rain_in = c.rain_in;
        out->source_in = c.source_in;
        out->evap_out = c.evap_out;
        out->outflow = c.outflow;
        out->clamp_gain = c.clamp_gain;
        out->q_out = c.q_out;
        out->s_max = c.s_max;
        out->dt_last = c.dt2;
        double inflow = out->rain_in + out->source_in;
        double resid = out->volume - out->volume0 - out->rain_in - out->source_in + out->evap_out + out->outflow;
        out->balance_error = resid / std::max(std::fabs(inflow), 1e-300);
        return SW2D_OK;
    }
    if (h->have_depth && (rc = prime(h, 1))) return rc; /* volume of the current state */
    DevClock c;
    if ((rc = read_clock(h, &c))) return rc;
    out->time = c.t;
    out->iterations = (double)c.iters;
    out->volume = c.led[LED_VOLUME];
    out->volume0 = c.led[LED_VOLUME0];
    out->rain_in = c.led[LED_RAIN];
    out->source_in = c.led[LED_SOURCE];
    out->evap_out = c.led[LED_EVAP];
    out->outflow = c.led[LED_OUTFLOW];
    out->clamp_gain = c.led[LED_CLAMP];
    out->q_out = c.led[LED_QOUT];
    out->s_max = c.led[LED_SMAX];
    out->dt_last = c.led[LED_DTLAST];
    double inflow = out->rain_in + out->source_in;
    double resid = out->volume - out->volume0 - out->rain_in - out->source_in + out->evap_out + out->outflow;
    out->balance_error = resid / std::max(std::fabs(inflow), 1e-300);
    return SW2D_OK;
}

int sw2d_set_outlet_record(sw2d_handle* h, int capacity) {
    if (!h || capacity < 0) return fail(SW2D_ERR_INVALID, "capacity");
    int rc = set_device(h);
    if (rc) return rc;
    if (h->fp32()) {
        h->outlet_cap = capacity;
        return h->have_depth ? fp32_rebuild(h) : SW2D_OK;
    }
    dfree(h->outlet);
    h->outlet_cap = 0;
    if (capacity > 0) {
        if ((rc = dalloc(&h->outlet, (size_t)capacity * 2))) return rc;
        h->outlet_cap = capacity;
    }
    long long zero_n = 0;
    if ((rc = put(h, &h->clk->outlet_n, &zero_n, sizeof zero_n))) return rc;
    h->graph_dirty = true;
    return SW2D_OK;
}

int sw2d_get_outlet(sw2d_handle* h, double* t, double* q, int capacity, int* count_out) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    int rc = set_device(h);
    if (rc) return rc;
    if (h->fp32()) {
        if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
        std::string err;
        if ((rc = h->eng->get_outlet(h->eng_idx, t, q, capacity, count_out, &err))) return fail(rc, err);
        return SW2D_OK;
    }
    DevClock c;
    if ((rc = read_clock(h, &c))) return rc;
    long long n = std::min<long long>(c.outlet_n, h->outlet_cap);
    if (count_out) *count_out = (int)n;
    if (n == 0 || (!t && !q)) return SW2D_OK;
    std::vector<double> buf((size_t)h->outlet_cap * 2);
    CK(cudaMemcpy(buf.data(), h->outlet, buf.size() * sizeof(double), cudaMemcpyDeviceToHost));
    long long first = c.outlet_n > h->outlet_cap ? c.outlet_n % h->outlet_cap : 0;
    for (long long k = 0; k < n && k < capacity; k++) {
        long long j = (first + k) % h->outlet_cap;
        if (t) t[k] = buf[2 * j];
        if (q) q[k] = buf[2 * j + 1];
    }
    return SW2D_OK;
}

int sw2d_set_profiling(sw2d_handle* h, int on) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    h->profiling = on != 0;
    h->kernel_ms.assign(8, 0.0);
    h->prof_iters = 0;
    return SW2D_OK;
}

int sw2d_get_timing(sw2d_handle* h, double* ms, double* kernel_ms, int* nk) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (h->fp32()) {
        if (ms) *ms = h->last_ms_per_iter;
        if (nk) *nk = 0;
        return SW2D_OK;
    }
    if (ms) *ms = h->last_ms_per_iter;
    const int n = fp64_kernels_per_iteration();
    if (nk) *nk = n;
    if (kernel_ms)
        for (int k = 0; k < n; k++) kernel_ms[k] = h->prof_iters ? h->kernel_ms[k] / h->prof_iters : 0.0;
    return SW2D_OK;
}

/* snapshot layout: a 64-byte header (magic, rows, cols, pitch, clock size),
 * the device clock, then the state arrays: FP64 h, qx, qy (padded); FP32 h,
 * qx, qy and the Kahan compensation (padded binary32) */
constexpr int64_t kSnapMagic64 = 0x53573244534e4150LL, kSnapMagic32 = 0x5357324433325350LL;

int sw2d_snapshot_size(sw2d_handle* h, size_t* bytes) {
    if (!h || !bytes) return fail(SW2D_ERR_INVALID, "null argument");
    if (h->fp32()) {
        if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
        *bytes = 64 + h->eng->snapshot_bytes(h->eng_idx);
        return SW2D_OK;
    }
    *bytes = 64 + sizeof(DevClock) + 3 * h->ncell * sizeof(double);
    return SW2D_OK;
}

static int snapshot_fp32(sw2d_handle* h, void* buf, size_t bytes) {
    size_t need;
    int rc = sw2d_snapshot_size(h, &need);
    if (rc) return rc;
    if (!buf || bytes < need) return fail(SW2D_ERR_INVALID, "snapshot buffer too small");
    const sw2d::Scenario32& S = h->eng->at(h->eng_idx);
    int64_t hdr[8] = {kSnapMagic32, h->R, h->C, S.P, (int64_t)sizeof(sw2d::Clock32), 0, 0, 0};
    std::memcpy(buf, hdr, 64);
    std::string err;
    if ((rc = h->eng->snapshot(h->eng_idx, (char*)buf + 64, &err))) return fail(rc, err);
    return SW2D_OK;
}

static int restore_fp32(sw2d_handle* h, const void* buf, size_t bytes) {
    if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
    size_t need;
    int rc = sw2d_snapshot_size(h, &need);
    if (rc) return rc;
    if (bytes < need) return fail(SW2D_ERR_INVALID, "snapshot too small");
    const sw2d::Scenario32& S = h->eng->at(h->eng_idx);
    int64_t hdr[8];
    std::memcpy(hdr, buf, 64);
    if (hdr[0] != kSnapMagic32 || hdr[1] != h->R || hdr[2] != h->C || hdr[3] != S.P ||
        hdr[4] != (int64_t)sizeof(sw2d::Clock32))
        return fail(SW2D_ERR_INVALID, "snapshot does not match this model");
    std::string err;
    if ((rc = h->eng->restore(h->eng_idx, (const char*)buf + 64, &err))) return fail(rc, err);
    return SW2D_OK;
}

int sw2d_snapshot(sw2d_handle* h, void* buf, size_t bytes) {
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->fp32()) return snapshot_fp32(h, buf, bytes);
    size_t need;
    sw2d_snapshot_size(h, &need);
    if (!buf || bytes < need) return fail(SW2D_ERR_INVALID, "snapshot buffer too small");
    char* p = (char*)buf;
    int64_t hdr[8] = {kSnapMagic64, h->R, h->C, h->P, (int64_t)sizeof(DevClock), 0, 0, 0};
    std::memcpy(p, hdr, 64);
    p += 64;
    CK(cudaMemcpy(p, h->clk, sizeof(DevClock), cudaMemcpyDeviceToHost));
    p += sizeof(DevClock);
    double* src[3] = {h->h[0], h->qx[0], h->qy[0]};
    for (int k = 0; k < 3; k++) {
        if ((rc = d2h(h, p, src[k], h->ncell * sizeof(double)))) return rc;
        p += h->ncell * sizeof(double);
    }
    return SW2D_OK;
}

int sw2d_restore(sw2d_handle* h, const void* buf, size_t bytes) {
    if (!h || !buf) return fail(SW2D_ERR_INVALID, "null argument");
    if (!h->have_dem) return fail(SW2D_ERR_STATE, "set_dem first");
    if (h->fp32()) {
        int rc = set_device(h);
        return rc ? rc : restore_fp32(h, buf, bytes);
    }
    int rc = set_device(h);
    if (rc) return rc;
    size_t need;
    sw2d_snapshot_size(h, &need);
    if (bytes < need) return fail(SW2D_ERR_INVALID, "snapshot too small");
    const char* p = (const char*)buf;
    int64_t hdr[8];
    std::memcpy(hdr, p, 64);
    if (hdr[0] != kSnapMagic64 || hdr[1] != h->R || hdr[2] != h->C || hdr[3] != h->P ||
        hdr[4] != (int64_t)sizeof(DevClock))
        return fail(SW2D_ERR_INVALID, "snapshot does not match this model");
    p += 64;
    DevClock c;
    std::memcpy(&c, p, sizeof c);
    c.counter = 0;
    if ((rc = put(h, h->clk, &c, sizeof c))) return rc;
    p += sizeof(DevClock);
    double* dst[3] = {h->h[0], h->qx[0], h->qy[0]};
    for (int k = 0; k < 3; k++) {
        if ((rc = put(h, dst[k], p, h->ncell * sizeof(double)))) return rc;
        p += h->ncell * sizeof(double);
    }
    h->have_depth = true;
    StepParams sp = h->params();
    fp64_launch_face_velocity(sp, 0, h->stream);
    if ((rc = sync_check(h))) return rc;
    return prime(h, 0);
}

int sw2d_test_stall_staging(sw2d_handle* h, int on) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    if (!h->fp32()) return fail(SW2D_ERR_STATE, "staging stall: FP32 handles only");
    if (h->eng_idx < 0) return fail(SW2D_ERR_STATE, "set_depth first");
    h->eng->set_stall_staging(h->eng_idx, on != 0);
    return SW2D_OK;
}

/* ---------------- coupling: SW2D-EFDC.cu:728-1067 ---------------------- */

}  /* extern "C" */

/* The boundary faces of a lake mask (1 = lake) as couple_BC_efdc finds them
 * (SW2D-EFDC.cu:739-1065): rows from the bottom (ini), columns left to
 * right, each non-lake cell testing south, north, east, west in that order;
 * edge rows and columns test only the sides the reference tests there,
 * corner cells none.  Side 0 N, 1 S, 2 E, 3 W; EFDC 1-based (I, J). */
static void scan_coupling_faces(int rows, int cols, const int* mask, std::vector<int>* side, std::vector<int>* fi,
                                std::vector<int>* fj, std::vector<int>* cell) {
    side->clear();
    fi->clear();
    fj->clear();
    cell->clear();
    auto add = [&](int sd, int i, int j, int p) {
        side->push_back(sd);
        fi->push_back(i);
        fj->push_back(j);
        cell->push_back(p);
    };
    for (int ini = 0; ini < rows; ini++) {
        int base = rows * cols - (ini + 1) * cols;
        for (int inj = 0; inj < cols; inj++) {
            int p = base + inj;
            if (mask[p] == 1) continue;
            bool S = false, N = false, E = false, W = false;
            if (ini > 0 && ini < rows - 1) {
                if (inj > 0 && inj < cols - 1) S = N = E = W = true;
                else if (inj == cols - 1) S = N = E = true;
                else if (inj == 0) S = N = W = true;
            }
            if (inj > 0 && inj < cols - 1) {
                if (ini == 0) S = E = W = true;
                else if (ini == rows - 1) N = E = W = true;
            }
            if (S && mask[p] != mask[p - cols]) add(1, inj + 1, ini + 2, p);
            if (N && mask[p] != mask[p + cols]) add(0, inj + 1, ini, p);
            if (E && mask[p] != mask[p - 1]) add(2, inj, ini + 1, p);
            if (W && mask[p] != mask[p + 1]) add(3, inj + 2, ini + 1, p);
        }
    }
}

extern "C" {

int sw2d_coupling_faces_of(int rows, int cols, const int* mask, int* side, int* efdc_i, int* efdc_j, int* cell,
                           int capacity, int* n_out) {
    if (!mask || rows < 1 || cols < 1 || capacity < 0) return fail(SW2D_ERR_INVALID, "invalid argument");
    if ((long long)rows * cols > (1LL << 30)) return fail(SW2D_ERR_INVALID, "raster too large");
    std::vector<int> sd, fi, fj, fc;
    scan_coupling_faces(rows, cols, mask, &sd, &fi, &fj, &fc);
    const int n = (int)sd.size();
    for (int k = 0; k < std::min(n, capacity); k++) {
        if (side) side[k] = sd[k];
        if (efdc_i) efdc_i[k] = fi[k];
        if (efdc_j) efdc_j[k] = fj[k];
        if (cell) cell[k] = fc[k];
    }
    if (n_out) *n_out = n;
    return SW2D_OK;
}

int sw2d_set_coupling_mask(sw2d_handle* h, const int* mask, int lagged, int* n_faces_out) {
    if (!h || !mask) return fail(SW2D_ERR_INVALID, "null argument");
    int rc = set_device(h);
    if (rc) return rc;
    const int cols = h->C;
    scan_coupling_faces(h->R, h->C, mask, &h->f_side, &h->f_i, &h->f_j, &h->f_cell);
    h->nfaces = (int)h->f_side.size();
    h->lagged = lagged ? 1 : 0;
    dfree(h->d_face);
    dfree(h->d_face_vel);
    dfree(h->d_face_q);
    /* the faces on the device: the FP64 kernel takes padded cell indices,
     * the FP32 kernel raster indices (its scenario has its own pitch) */
    std::vector<int> dev((size_t)h->nfaces * 2 + 2);
    for (int k = 0; k < h->nfaces; k++) {
        int p = h->f_cell[k];
        dev[2 * k] = h->fp32() ? p : (int)h->pad_index(p / cols, p % cols);
        dev[2 * k + 1] = h->f_side[k];
    }
    if ((rc = dalloc(&h->d_face, dev.size()))) return rc;
    if ((rc = dalloc(&h->d_face_vel, (size_t)h->nfaces + 1))) return rc;
    if ((rc = dalloc(&h->d_face_q, (size_t)h->nfaces + 1))) return rc;
    CK(cudaMemcpy(h->d_face, dev.data(), dev.size() * sizeof(int), cudaMemcpyHostToDevice));
    if (n_faces_out) *n_faces_out = h->nfaces;
    return SW2D_OK;
}

int sw2d_get_coupling_faces(sw2d_handle* h, int* side, int* fi, int* fj, int* cell, int capacity) {
    if (!h) return fail(SW2D_ERR_INVALID, "null handle");
    int n = std::min(capacity, h->nfaces);
    for (int k = 0; k < n; k++) {
        if (side) side[k] = h->f_side[k];
        if (fi) fi[k] = h->f_i[k];
        if (fj) fj[k] = h->f_j[k];
        if (cell) cell[k] = h->f_cell[k];
    }
    return SW2D_OK;
}

} /* extern "C" */

namespace sw2d {
void launch_couple(const StepParams& p, int nfaces, const int* faces, int lagged, int initial, double* vel_prev,
                   double* q, cudaStream_t s);
}

/* Boundary-discharge sample of an FP32 handle: the k_couple rule on the
 * scenario's device state (k32_couple), on the engine's stream. */
static int couple_sample_fp32(sw2d_handle* h, int initial, double* q_out, int capacity) {
    const sw2d::Scn32* d = h->eng->device_scenario(h->eng_idx);
    if (!d) return fail(SW2D_ERR_CUDA, "FP32 scenario descriptor");
    cudaStream_t st = h->eng->stream();
    sw2d::fp32_launch_couple(d, h->nfaces, h->d_face, h->lagged, initial, h->cfg.th, h->d_face_vel, h->d_face_q, st);
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    if (q_out) {
        int n = std::min(capacity, h->nfaces);
        CK(cudaMemcpy(q_out, h->d_face_q, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return SW2D_OK;
}

extern "C" int sw2d_couple_sample(sw2d_handle* h, int initial, double* q_out, int capacity) {
    sw2d::NvtxRange r("sw2d_couple_sample");
    int rc = check_ready(h);
    if (rc) return rc;
    if (h->nfaces == 0) return SW2D_OK;
    if (h->fp32()) return couple_sample_fp32(h, initial, q_out, capacity);
    StepParams p = h->params();
    sw2d::launch_couple(p, h->nfaces, h->d_face, h->lagged, initial, h->d_face_vel, h->d_face_q, h->stream);
    if ((rc = sync_check(h))) return rc;
    if (q_out) {
        int n = std::min(capacity, h->nfaces);
        CK(cudaMemcpy(q_out, h->d_face_q, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return SW2D_OK;
}
