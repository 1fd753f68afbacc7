/* Host engine of the FP32 precision form (see sw2d_engine.h). */
#include "sw2d_engine.h"

#include <cudaTypedefs.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <limits>

namespace sw2d {

namespace {


PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void* p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

bool make_map(CUtensorMap* tm, void* base, CUtensorMapDataType dt, size_t esize, uint64_t width, uint64_t height,
              uint32_t boxw, uint32_t boxh, bool nan_fill) {
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {width, height};
    cuuint64_t strides[1] = {width * esize};
    cuuint32_t box[2] = {boxw, boxh};
    cuuint32_t es[2] = {1, 1};
    return fn(tm, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              nan_fill ? CU_TENSOR_MAP_FLOAT_OOB_FILL_NAN_REQUEST_ZERO_FMA : CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
}

int pitch_of(int cols) { return ((cols + 12 + 31) / 32) * 32; }

#define ECK(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            if (err) *err = std::string(#call) + ": " + cudaGetErrorString(e_);     \
            return e_ == cudaErrorMemoryAllocation ? SW2D_ERR_NOMEM : SW2D_ERR_CUDA; \
        }                                                                           \
    } while (0)

} // namespace

Engine32::Engine32(int device) : device_(device) {}

Engine32::~Engine32() {
    cudaSetDevice(device_);
    if (stream_) cudaStreamSynchronize(stream_);
    for (auto& s : scn_)
        for (void* p : s->allocs) cudaFree(p);
    if (graph_) cudaGraphExecDestroy(graph_);
    cudaFree(d_scn_);
    cudaFree(d_work_);
    cudaFree(d_part_);
    cudaFree(d_ctl_);
    cudaFree(d_tmp_);
    if (ev_a_) cudaEventDestroy(ev_a_);
    if (ev_b_) cudaEventDestroy(ev_b_);
    if (ev_t0_) cudaEventDestroy(ev_t0_);
    if (ev_t1_) cudaEventDestroy(ev_t1_);
    if (stream_) cudaStreamDestroy(stream_);
    if (pin_) cudaFreeHost(pin_);
}

int Engine32::init(std::string* err) {
    ECK(cudaSetDevice(device_));
    ECK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    ECK(cudaEventCreate(&ev_a_));
    ECK(cudaEventCreate(&ev_b_));
    ECK(cudaMalloc(&d_tmp_, fp32_volume_scratch_bytes()));
    if (fp32_configure_kernels() != 0) {
        if (err) *err = "cannot enable the FP32 kernel's shared memory";
        return SW2D_ERR_CUDA;
    }
    /* rows per work item: SW2D_SEGMENT_ROWS fixes it (else the autotuner) */
    if (seg_fixed_ == 0) {
        if (const char* e = std::getenv("SW2D_SEGMENT_ROWS")) {
            const int v = std::atoi(e);
            if (v >= 16 && v <= M_MAXSEG) seg_ = seg_fixed_ = v;
        }
    }
    ECK(cudaEventCreate(&ev_t0_));
    ECK(cudaEventCreate(&ev_t1_));
    ECK(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, device_));
    for (int k = 0; k < T32_NCLASS; k++) {
        bps_[k] = fp32_blocks_per_sm(k);
        if (bps_[k] <= 0) {
            if (err) *err = "the FP32 kernel does not fit on an SM";
            return SW2D_ERR_CUDA;
        }
    }
    if (!encode_fn()) {
        if (err) *err = "cuTensorMapEncodeTiled unavailable";
        return SW2D_ERR_CUDA;
    }
    return SW2D_OK;
}

size_t Engine32::scenario_bytes(int rows, int cols, bool rain_field, int outlet_cap) {
    const size_t P = pitch_of(cols), NR = rows + 2 * M_H;
    const size_t cells = P * NR;
    size_t b = cells * (8 * sizeof(float) + 1); /* 8 float fields + optional Manning class byte */
    if (rain_field) b += cells * sizeof(float);
    const size_t tiles = (size_t)((cols + M_CW - 1) / M_CW) * ((rows + 15) / 16);
    b += tiles * sizeof(float) + (size_t)outlet_cap * 16 + sizeof(Clock32) + 4096;
    return b;
}

size_t Engine32::bytes_in_use() const {
    size_t b = 0;
    for (auto& s : scn_) b += s->bytes;
    return b;
}

int Engine32::add(const ScenarioInput& in, long long id, std::string* err, int* index_out) {
    ECK(cudaSetDevice(device_));
    if (in.rows < 2 || in.cols < 2 || !in.dem) {
        if (err) *err = "scenario needs rows, cols >= 2 and a DEM";
        return SW2D_ERR_INVALID;
    }
    if (in.mclass && (in.ntable <= 0 || in.ntable > T32_MAXCLASS || !in.mtable)) {
        if (err) *err = "Manning table must have 1..64 entries";
        return SW2D_ERR_INVALID;
    }
    auto sp = std::make_unique<Scenario32>();
    Scenario32& S = *sp;
    S.id = id;
    const int R = in.rows, C = in.cols, P = pitch_of(C), NR = R + 2 * M_H;
    S.R = R;
    S.C = C;
    S.P = P;
    S.NR = NR;
    const size_t cells = (size_t)P * NR;
    const int tx = (C + M_CW - 1) / M_CW, nb = (R + M_DR - 1) / M_DR; /* datum tiles: strips x bands */
    auto alloc = [&](size_t bytes, void** p) -> int {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
        if (e != cudaSuccess) {
            if (err) *err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
            return SW2D_ERR_NOMEM;
        }
        S.allocs.push_back(*p);
        S.bytes += bytes;
        cudaMemsetAsync(*p, 0, std::max<size_t>(bytes, 16), stream_);
        return SW2D_OK;
    };
    auto fail_free = [&](int rc) {
        cudaStreamSynchronize(stream_);
        for (void* p : S.allocs) cudaFree(p);
        return rc;
    };
    Scn32& d = S.d;
    void* p;
    int rc;
    for (int k = 0; k < 2; k++) {
        if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
        d.h[k] = (float*)p;
        if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
        d.qx[k] = (float*)p;
        if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
        d.qy[k] = (float*)p;
    }
    if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
    d.kc = (float*)p;
    float* dz;
    if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
    dz = (float*)p;
    d.z = dz;
    uint8_t* dcls = nullptr;
    if (in.mclass) {
        if ((rc = alloc(cells, &p))) return fail_free(rc);
        dcls = (uint8_t*)p;
    }
    d.cls = dcls;
    float* ddatum;
    if ((rc = alloc((size_t)tx * nb * 4, &p))) return fail_free(rc);
    ddatum = (float*)p;
    d.datum = ddatum;
    float* drw = nullptr;
    if (in.rain_weight) {
        if ((rc = alloc(cells * 4, &p))) return fail_free(rc);
        drw = (float*)p;
    }
    d.rainw = drw;
    const int nrain = std::max(in.nrain, 1);
    double* drain;
    if ((rc = alloc((size_t)(nrain + 2) * 8, &p))) return fail_free(rc);
    drain = (double*)p;
    d.rain = drain;
    /* evaporation series and point sources (a later source on a cell
     * replaces an earlier one, as the reference's stream_flow writes them) */
    double* devap = nullptr;
    if (in.evap && in.nevap > 0) {
        if ((rc = alloc((size_t)(in.nevap + 2) * 8, &p))) return fail_free(rc);
        devap = (double*)p;
    }
    std::vector<int> src_keep;
    if (in.nsrc > 0) {
        if (in.nsrc > T32_MAXSRC || !in.src_cells || !in.src_q || in.nq <= 0 || !(in.dtoq > 0)) {
            if (err) *err = "point sources";
            return fail_free(SW2D_ERR_INVALID);
        }
        for (int k = 0; k < in.nsrc; k++) {
            if (in.src_cells[k] < 0 || in.src_cells[k] >= R * C) {
                if (err) *err = "source cell out of range";
                return fail_free(SW2D_ERR_INVALID);
            }
            bool later = false;
            for (int j = k + 1; j < in.nsrc; j++) later |= in.src_cells[j] == in.src_cells[k];
            if (!later) src_keep.push_back(k);
        }
    }
    const int nu = (int)src_keep.size();
    int* dsrc_cell = nullptr;
    double* dsrcq = nullptr;
    if (nu > 0) {
        if ((rc = alloc((size_t)nu * 4, &p))) return fail_free(rc);
        dsrc_cell = (int*)p;
        if ((rc = alloc((size_t)(in.nq + 2) * nu * 8, &p))) return fail_free(rc);
        dsrcq = (double*)p;
    }
    d.evap = devap;
    d.srcq = dsrcq;
    d.src_cell = dsrc_cell;
    d.outlet = nullptr;
    if (in.outlet_cap > 0) {
        if ((rc = alloc((size_t)in.outlet_cap * 16, &p))) return fail_free(rc);
        d.outlet = (double*)p;
    }
    Clock32* dclk;
    if ((rc = alloc(sizeof(Clock32), &p))) return fail_free(rc);
    dclk = (Clock32*)p;
    d.clk = dclk;

    /* host staging: per datum tile (a strip of 224 columns x a band of 64
     * rows) the mean active elevation rounded to 1/16 m, bed offsets from it
     * with NaN for inactive cells */
    std::vector<float> datum((size_t)tx * nb, 0.f);
    std::vector<float> zoff(cells, std::numeric_limits<float>::quiet_NaN()), hbuf(cells, 0.f), rw;
    std::vector<uint8_t> cls;
    if (in.mclass) cls.assign(cells, 0);
    double active_weight = 0.0;
    for (int j = 0; j < nb; j++)
        for (int i = 0; i < tx; i++) {
            double sum = 0;
            long n = 0;
            for (int r = j * M_DR; r < std::min(R, (j + 1) * M_DR); r++)
                for (int c = i * M_CW; c < std::min(C, (i + 1) * M_CW); c++) {
                    double z = in.dem[(size_t)r * C + c];
                    if (z != in.nodata) {
                        sum += z;
                        n++;
                    }
                }
            datum[(size_t)j * tx + i] = n ? (float)(std::round(sum / n * 16.0) / 16.0) : 0.f;
        }
    if (in.rain_weight) rw.assign(cells, 1.f);
    for (int r = 0; r < R; r++)
        for (int c = 0; c < C; c++) {
            const size_t k = (size_t)r * C + c;
            const size_t g = (size_t)(r + M_H) * P + (c + M_H);
            const double z = in.dem[k];
            const bool act = z != in.nodata;
            const double dat = datum[(size_t)(r / M_DR) * tx + (c / M_CW)];
            if (act) zoff[g] = (float)(z - dat);
            if (in.mclass) {
                const uint8_t cl = in.mclass[k];
                if (cl >= in.ntable) {
                    if (err) *err = "Manning class out of table range";
                    return fail_free(SW2D_ERR_INVALID);
                }
                cls[g] = cl;
            }
            hbuf[g] = (act && in.depth) ? (float)in.depth[k] : 0.f;
            if (in.rain_weight) rw[g] = in.rain_weight[k];
            if (act) active_weight += in.rain_weight ? (double)in.rain_weight[k] : 1.0;
        }
    ECK(cudaMemcpyAsync(dz, zoff.data(), cells * 4, cudaMemcpyHostToDevice, stream_));
    if (dcls) ECK(cudaMemcpyAsync(dcls, cls.data(), cells, cudaMemcpyHostToDevice, stream_));
    ECK(cudaMemcpyAsync(d.h[0], hbuf.data(), cells * 4, cudaMemcpyHostToDevice, stream_));
    ECK(cudaMemcpyAsync(ddatum, datum.data(), datum.size() * 4, cudaMemcpyHostToDevice, stream_));
    if (drw) ECK(cudaMemcpyAsync(drw, rw.data(), cells * 4, cudaMemcpyHostToDevice, stream_));
    std::vector<double> rain(nrain + 2, 0.0);
    for (int k = 0; k < in.nrain; k++) rain[k] = in.rain[k];
    ECK(cudaMemcpyAsync(drain, rain.data(), rain.size() * 8, cudaMemcpyHostToDevice, stream_));
    std::vector<double> evap, srcq;
    std::vector<int> srcc;
    if (devap) {
        evap.assign((size_t)in.nevap + 2, 0.0);
        for (int k = 0; k < in.nevap; k++) evap[k] = in.evap[k];
        ECK(cudaMemcpyAsync(devap, evap.data(), evap.size() * 8, cudaMemcpyHostToDevice, stream_));
    }
    if (nu > 0) {
        srcq.assign((size_t)(in.nq + 2) * nu, 0.0);
        for (int u = 0; u < nu; u++) {
            srcc.push_back(in.src_cells[src_keep[u]]);
            for (int t = 0; t < in.nq; t++) srcq[(size_t)t * nu + u] = in.src_q[(size_t)t * in.nsrc + src_keep[u]];
        }
        ECK(cudaMemcpyAsync(dsrc_cell, srcc.data(), srcc.size() * 4, cudaMemcpyHostToDevice, stream_));
        ECK(cudaMemcpyAsync(dsrcq, srcq.data(), srcq.size() * 8, cudaMemcpyHostToDevice, stream_));
    }

    /* tensor maps: rows of 232 columns, four rows per staged block; the bed
     * reads NaN (inactive) outside the array */
    bool ok = true;
    for (int k = 0; k < 2; k++) {
        ok &= make_map(&d.tm_h[k], d.h[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RB, false);
        ok &= make_map(&d.tm_qx[k], d.qx[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RB, false);
        ok &= make_map(&d.tm_qy[k], d.qy[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RB, false);
    }
    ok &= make_map(&d.tm_z, dz, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RB, true);
    ok &= make_map(&d.tm_kc, d.kc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RB, false);
    if (dcls) ok &= make_map(&d.tm_cls, dcls, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, P, NR, M_CLSW, M_CLSR, false);
    if (drw) ok &= make_map(&d.tm_rw, drw, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, P, NR, M_BW, M_RWR, false);
    if (!ok) {
        if (err) *err = "cuTensorMapEncodeTiled failed";
        return fail_free(SW2D_ERR_CUDA);
    }
    d.R = R;
    d.C = C;
    d.P = P;
    d.tiles_x = tx;
    d.bands = nb;
    d.seg = 0;     /* work items: set by rebuild */
    d.tiles_y = 0;
    d.outflow_south = in.outflow_south;
    d.series_mode = in.series_mode;
    d.dt_mode = in.dt_mode;
    d.nrain = nrain;
    d.nevap = devap ? in.nevap : 0;
    d.nsrc = nu;
    d.nq = nu > 0 ? in.nq : 0;
    d.dtoq = nu > 0 ? in.dtoq : 3600.0;
    d.outlet_cap = in.outlet_cap;
    d.dx = (float)in.dx;
    d.dy = (float)in.dy;
    d.rdx = (float)(1.0 / in.dx);
    d.rdy = (float)(1.0 / in.dy);
    d.th = (float)in.th;
    d.g = (float)in.g;
    const double pct_lake = 1.00 - in.frac_lwl, pct_land = 1.00 - (in.frac_int + in.frac_inf);
    d.pct_lake = (float)pct_lake;
    d.pct_land = (float)pct_land;
    d.ev_wl_min = (float)in.ev_wl_min;
    d.ledger_cells = pct_lake != pct_land || devap != nullptr; /* evaporation acts on lake cells only */
    d.rain_static = active_weight * pct_land;
    d.dxd = in.dx;
    d.dyd = in.dy;
    d.dtrain = in.dtrain;
    d.dt_fixed = in.dt;
    d.cfl = in.cfl;
    d.dt_max = in.dt_max;
    d.area = in.dx * in.dy;
    for (int k = 0; k < T32_MAXCLASS; k++)
        d.ntab[k] = (float)(in.mclass ? (k < in.ntable ? in.mtable[k] : 0.0) : in.manning);
    Clock32 c{};
    c.t = in.t0;
    c.t_end = in.t_end;
    ECK(cudaMemcpyAsync(dclk, &c, sizeof c, cudaMemcpyHostToDevice, stream_));
    ECK(cudaStreamSynchronize(stream_));
    S.t_end_default = in.t_end;
    scn_.push_back(std::move(sp));
    const int idx = (int)scn_.size() - 1;
    dirty_ = true;
    if ((rc = rebuild(err))) return rc;
    /* initial volume and CFL speed, then the first slot */
    fp32_launch_volume(d_scn_, idx, scn_[idx]->d, d_tmp_, stream_);
    double vs[2];
    ECK(cudaMemcpyAsync(vs, d_tmp_, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    ECK(cudaStreamSynchronize(stream_));
    c.volume0 = vs[0];
    c.s_max = vs[1];
    ECK(cudaMemcpyAsync(dclk, &c, sizeof c, cudaMemcpyHostToDevice, stream_));
    fp32_launch_prime(d_scn_ + idx, 1, stream_);
    ECK(cudaStreamSynchronize(stream_));
    ECK(cudaGetLastError());
    if (index_out) *index_out = idx;
    return SW2D_OK;
}

int Engine32::remove(int index) {
    if (index < 0 || index >= (int)scn_.size()) return SW2D_ERR_INVALID;
    cudaSetDevice(device_);
    cudaStreamSynchronize(stream_);
    for (void* p : scn_[index]->allocs) cudaFree(p);
    scn_.erase(scn_.begin() + index);
    dirty_ = true;
    return SW2D_OK;
}

int Engine32::rebuild(std::string* err) {
    if (!dirty_) return SW2D_OK;
    work_.clear();
    std::vector<Scn32> host(scn_.size());
    /* work items grouped by feature class, scenarios in order within a class;
     * .w is the item's slot in the scenario-ordered partials */
    for (int k = 0; k < T32_NCLASS; k++) {
        class_first_[k] = (int)work_.size();
        for (size_t i = 0; i < scn_.size(); i++) {
            Scn32& d = scn_[i]->d;
            if (fp32_feature_class(d) != k) continue;
            d.seg = std::min(seg_, d.R);
            d.tiles_y = (d.R + d.seg - 1) / d.seg;
            d.first_work = (int)work_.size();
            for (int ty = 0; ty < d.tiles_y; ty++)
                for (int tx = 0; tx < d.tiles_x; tx++)
                    work_.push_back(make_int4((int)i, tx, ty, (int)work_.size()));
            d.nwork = (int)work_.size() - d.first_work;
            host[i] = d;
        }
        class_n_[k] = (int)work_.size() - class_first_[k];
        /* the class's longest items first in every iteration (a scenario's
         * last segment is shorter), so the tail of an iteration holds short
         * items; the order is the same in every iteration, so a scenario's
         * items of the next iteration come after its own of this one */
        auto rows_of = [&](const int4& w) {
            const Scn32& d = scn_[w.x]->d;
            return std::min(d.seg, d.R - w.z * d.seg);
        };
        std::stable_sort(work_.begin() + class_first_[k], work_.end(),
                         [&](const int4& a, const int4& b) { return rows_of(a) > rows_of(b); });
    }
    if (host.size() > d_scn_cap_) {
        cudaFree(d_scn_);
        d_scn_ = nullptr;
        d_scn_cap_ = std::max<size_t>(host.size(), 2 * d_scn_cap_);
        ECK(cudaMalloc(&d_scn_, d_scn_cap_ * sizeof(Scn32)));
    }
    if (work_.size() > d_work_cap_) {
        cudaFree(d_work_);
        cudaFree(d_part_);
        d_work_ = nullptr;
        d_part_ = nullptr;
        d_work_cap_ = std::max<size_t>(work_.size(), 2 * d_work_cap_);
        ECK(cudaMalloc(&d_work_, d_work_cap_ * sizeof(int4)));
        ECK(cudaMalloc(&d_part_, d_work_cap_ * sizeof(Part32)));
    }
    if (fp32_ctl_bytes((int)scn_.size()) > d_ctl_cap_) {
        cudaFree(d_ctl_);
        d_ctl_ = nullptr;
        d_ctl_cap_ = std::max(fp32_ctl_bytes((int)scn_.size()), 2 * d_ctl_cap_);
        ECK(cudaMalloc(&d_ctl_, d_ctl_cap_));
    }
    if (!host.empty())
        ECK(cudaMemcpyAsync(d_scn_, host.data(), host.size() * sizeof(Scn32), cudaMemcpyHostToDevice, stream_));
    if (!work_.empty())
        ECK(cudaMemcpyAsync(d_work_, work_.data(), work_.size() * sizeof(int4), cudaMemcpyHostToDevice, stream_));
    ECK(cudaStreamSynchronize(stream_));
    if (graph_) {
        cudaGraphExecDestroy(graph_);
        graph_ = nullptr;
    }
    dirty_ = false;
    return SW2D_OK;
}

/* CTAs of class k's persistent launch over niter iterations: the CTAs per
 * SM in use (at most what the SM holds) on every SM, at most one per queue
 * ticket */
int Engine32::grid_of(int k, int niter) const {
    const int per_sm = cps_ > 0 ? std::min(cps_, bps_[k]) : bps_[k];
    return (int)std::max<long long>(1, std::min<long long>((long long)per_sm * nsm_, (long long)class_n_[k] * niter));
}

/* niter iterations: one persistent launch per feature class present */
int Engine32::launch(int niter, std::string* err) {
    int grid[T32_NCLASS];
    for (int k = 0; k < T32_NCLASS; k++) grid[k] = grid_of(k, niter);
    ECK(fp32_launch_chunk(d_scn_, (int)scn_.size(), d_work_, class_first_, class_n_, d_part_, d_ctl_, niter, grid,
                          stream_));
    return SW2D_OK;
}

int Engine32::build_graph(std::string* err) {
    if (graph_ || graph_failed_) return SW2D_OK;
    cudaGraph_t g = nullptr;
    ECK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    int grid[T32_NCLASS];
    for (int k = 0; k < T32_NCLASS; k++) grid[k] = grid_of(k, kChunk);
    cudaError_t el = fp32_launch_chunk(d_scn_, (int)scn_.size(), d_work_, class_first_, class_n_, d_part_, d_ctl_, kChunk,
                                       grid, stream_);
    cudaError_t ec = cudaStreamEndCapture(stream_, &g);
    cudaError_t ei = cudaErrorUnknown;
    if (el == cudaSuccess && ec == cudaSuccess && g) ei = cudaGraphInstantiate(&graph_, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        /* a cooperative launch the capture could not take: the chunks are
         * launched directly (one launch per 32 iterations either way) */
        graph_ = nullptr;
        graph_failed_ = true;
        cudaGetLastError();
    }
    return SW2D_OK;
}

int Engine32::tune(long long budget, std::string* err, long long* advanced) {
    *advanced = 0;
    double cells = 0;
    for (auto& sp : scn_) cells += (double)sp->R * sp->C;
    if (seg_fixed_ > 0 || cells < (1 << 20)) return SW2D_OK;
    const int bucket = (int)std::floor(std::log2(cells));
    if (bucket == bucket_) return SW2D_OK;
    int rc;
    auto use = [&](int seg, int cps) {
        if (seg != seg_ || cps != cps_) {
            seg_ = seg;
            cps_ = cps;
            dirty_ = true; /* new work items, and the chunk graph holds the grid */
            return rebuild(err);
        }
        return (int)SW2D_OK;
    };
    const auto cached = tuned_.find(bucket);
    if (cached != tuned_.end()) {
        if ((rc = use(cached->second.first, cached->second.second))) return rc;
        bucket_ = bucket;
        return SW2D_OK;
    }
    int most = 0;
    for (int k = 0; k < T32_NCLASS; k++)
        if (class_n_[k] > 0) most = std::max(most, bps_[k]);
    std::vector<std::pair<int, int>> cands;
    for (int seg : {64, 128, 256, 512}) {
        cands.emplace_back(seg, 0);
        if (most > 1) cands.emplace_back(seg, most - 1);
    }
    /* iterations per candidate: one untimed (the new work split's first
     * launch), then one timed launch of up to a chunk */
    const long long per = std::min<long long>(kChunk + 1, budget / (long long)cands.size());
    if (per < 3) return SW2D_OK; /* too few iterations to tune now: a later, longer call will */
    const auto t0 = std::chrono::steady_clock::now();
    std::pair<int, int> best(seg_, cps_);
    float best_ms = 3.4e38f;
    for (const auto& cand : cands) {
        if ((rc = use(cand.first, cand.second))) return rc;
        if ((rc = launch(1, err))) return rc;
        ECK(cudaEventRecord(ev_t0_, stream_));
        if ((rc = launch((int)(per - 1), err))) return rc;
        ECK(cudaEventRecord(ev_t1_, stream_));
        ECK(cudaEventSynchronize(ev_t1_));
        float ms = 0;
        ECK(cudaEventElapsedTime(&ms, ev_t0_, ev_t1_));
        *advanced += per;
        if (ms < best_ms) {
            best_ms = ms;
            best = cand;
        }
    }
    if ((rc = use(best.first, best.second))) return rc;
    tuned_[bucket] = best;
    bucket_ = bucket;
    tuning_ms_ += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    tunings_++;
    return SW2D_OK;
}

int Engine32::tune_now(long long budget, std::string* err, long long* advanced) {
    ECK(cudaSetDevice(device_));
    *advanced = 0;
    int rc = rebuild(err);
    if (rc) return rc;
    if (scn_.empty() || budget <= 0) return SW2D_OK;
    return tune(budget, err, advanced);
}

int Engine32::set_t_end(int index, double t_end, std::string* err) {
    ECK(cudaSetDevice(device_));
    for (int i = 0; i < (int)scn_.size(); i++) {
        if (index >= 0 && i != index) continue;
        ECK(cudaMemcpyAsync(&scn_[i]->d.clk->t_end, &t_end, sizeof(double), cudaMemcpyHostToDevice, stream_));
        ECK(cudaStreamSynchronize(stream_));
    }
    int rc = rebuild(err);
    if (rc) return rc;
    if (index >= 0)
        fp32_launch_prime(d_scn_ + index, 1, stream_);
    else if (!scn_.empty())
        fp32_launch_prime(d_scn_, (int)scn_.size(), stream_);
    ECK(cudaStreamSynchronize(stream_));
    return SW2D_OK;
}

int Engine32::run(long long n, std::string* err) {
    ECK(cudaSetDevice(device_));
    int rc = rebuild(err);
    if (rc) return rc;
    if (scn_.empty() || n <= 0) return SW2D_OK;
    ECK(cudaEventRecord(ev_a_, stream_));
    long long done = 0;
    if ((rc = tune(n, err, &done))) return rc;
    if ((rc = build_graph(err))) return rc;
    for (; n - done >= kChunk; done += kChunk) {
        if (graph_)
            ECK(cudaGraphLaunch(graph_, stream_));
        else if ((rc = launch(kChunk, err)))
            return rc;
    }
    if (n > done && (rc = launch((int)(n - done), err))) return rc;
    ECK(cudaGetLastError());
    ECK(cudaEventRecord(ev_b_, stream_));
    ECK(cudaEventSynchronize(ev_b_));
    float ms = 0;
    ECK(cudaEventElapsedTime(&ms, ev_a_, ev_b_));
    last_ms_ = ms;
    last_iters_ = n;
    return SW2D_OK;
}

int Engine32::sync(std::string* err) {
    ECK(cudaStreamSynchronize(stream_));
    return SW2D_OK;
}

int Engine32::get_clock(int index, Clock32* out, std::string* err) {
    ECK(cudaMemcpyAsync(out, scn_[index]->d.clk, sizeof(Clock32), cudaMemcpyDeviceToHost, stream_));
    ECK(cudaStreamSynchronize(stream_));
    return SW2D_OK;
}

int Engine32::get_state(int index, double* depth, double* qx, double* qy, std::string* err) {
    Scenario32& S = *scn_[index];
    Clock32 c;
    int rc = get_clock(index, &c, err);
    if (rc) return rc;
    const int cur = c.slot.cur;
    const int R = S.R, C = S.C, P = S.P;
    /* whole padded rows into pinned staging (a copy into pageable memory runs
     * at a few GB/s), then the interior widened to binary64 on host threads */
    const size_t need = (size_t)(R + 1) * P * sizeof(float);
    if (pin_bytes_ < need) {
        if (pin_) cudaFreeHost(pin_);
        pin_ = nullptr;
        pin_bytes_ = 0;
        ECK(cudaMallocHost(&pin_, need));
        pin_bytes_ = need;
    }
    auto fetch = [&](const float* src, int rows, int cols, double* dst) -> int {
        ECK(cudaMemcpyAsync(pin_, src + (size_t)M_H * P, (size_t)rows * P * sizeof(float), cudaMemcpyDeviceToHost,
                            stream_));
        ECK(cudaStreamSynchronize(stream_));
        const float* s = static_cast<const float*>(pin_) + M_H;
        const size_t nt = std::max<size_t>(1, std::min<size_t>({16, std::thread::hardware_concurrency(),
                                                                (size_t)rows / 64 + 1}));
        std::vector<std::thread> th;
        const size_t per = ((size_t)rows + nt - 1) / nt;
        for (size_t t = 0; t < nt; t++) {
            const size_t a = t * per, b = std::min((size_t)rows, a + per);
            if (a >= b) continue;
            th.emplace_back([=] {
                for (size_t r = a; r < b; r++)
                    for (int k = 0; k < cols; k++) dst[r * cols + k] = s[r * P + k];
            });
        }
        for (auto& x : th) x.join();
        return SW2D_OK;
    };
    if (depth && (rc = fetch(S.d.h[cur], R, C, depth))) return rc;
    if (qx && (rc = fetch(S.d.qx[cur], R + 1, C, qx))) return rc;
    if (qy && (rc = fetch(S.d.qy[cur], R, C + 1, qy))) return rc;
    return SW2D_OK;
}

size_t Engine32::snapshot_bytes(int index) const {
    const Scenario32& S = *scn_[index];
    return sizeof(Clock32) + 4 * (size_t)S.P * S.NR * sizeof(float);
}

int Engine32::snapshot(int index, void* buf, std::string* err) {
    Scenario32& S = *scn_[index];
    Clock32 c;
    int rc = get_clock(index, &c, err);
    if (rc) return rc;
    char* p = static_cast<char*>(buf);
    std::memcpy(p, &c, sizeof c);
    p += sizeof c;
    const size_t n = (size_t)S.P * S.NR * sizeof(float);
    const float* src[4] = {S.d.h[c.slot.cur], S.d.qx[c.slot.cur], S.d.qy[c.slot.cur], S.d.kc};
    for (int k = 0; k < 4; k++) {
        ECK(cudaMemcpyAsync(p, src[k], n, cudaMemcpyDeviceToHost, stream_));
        p += n;
    }
    ECK(cudaStreamSynchronize(stream_));
    return SW2D_OK;
}

int Engine32::restore(int index, const void* buf, std::string* err) {
    Scenario32& S = *scn_[index];
    const char* p = static_cast<const char*>(buf);
    Clock32 c;
    std::memcpy(&c, p, sizeof c);
    p += sizeof c;
    if (c.slot.cur != 0 && c.slot.cur != 1) {
        if (err) *err = "snapshot clock is not valid";
        return SW2D_ERR_INVALID;
    }
    const size_t n = (size_t)S.P * S.NR * sizeof(float);
    float* dst[4] = {S.d.h[c.slot.cur], S.d.qx[c.slot.cur], S.d.qy[c.slot.cur], S.d.kc};
    for (int k = 0; k < 4; k++) {
        ECK(cudaMemcpyAsync(dst[k], p, n, cudaMemcpyHostToDevice, stream_));
        p += n;
    }
    ECK(cudaMemcpyAsync(S.d.clk, &c, sizeof c, cudaMemcpyHostToDevice, stream_));
    ECK(cudaStreamSynchronize(stream_));
    return SW2D_OK;
}

int Engine32::get_volume(int index, double* vol, double* smax, std::string* err) {
    int rc = rebuild(err);
    if (rc) return rc;
    fp32_launch_volume(d_scn_, index, scn_[index]->d, d_tmp_, stream_);
    double vs[2];
    ECK(cudaMemcpyAsync(vs, d_tmp_, 2 * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    ECK(cudaStreamSynchronize(stream_));
    if (vol) *vol = vs[0];
    if (smax) *smax = vs[1];
    return SW2D_OK;
}

int Engine32::get_outlet(int index, double* t, double* q, int cap, int* count, std::string* err) {
    Scenario32& S = *scn_[index];
    Clock32 c;
    int rc = get_clock(index, &c, err);
    if (rc) return rc;
    const int oc = S.d.outlet_cap;
    long long n = std::min<long long>(c.outlet_n, oc);
    if (count) *count = (int)n;
    if (!n || (!t && !q)) return SW2D_OK;
    std::vector<double> buf((size_t)oc * 2);
    ECK(cudaMemcpyAsync(buf.data(), S.d.outlet, buf.size() * 8, cudaMemcpyDeviceToHost, stream_));
    ECK(cudaStreamSynchronize(stream_));
    long long first = c.outlet_n > oc ? c.outlet_n % oc : 0;
    for (long long k = 0; k < n && k < cap; k++) {
        long long j = (first + k) % oc;
        if (t) t[k] = buf[2 * j];
        if (q) q[k] = buf[2 * j + 1];
    }
    return SW2D_OK;
}

} // namespace sw2d
