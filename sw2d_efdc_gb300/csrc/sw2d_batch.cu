/* Batched and served FP32 SW2D: many scenarios of uneven raster sizes
 * advanced together by the row-marching kernel (per iteration, one launch
 * per feature class present over its part of a work list of (scenario,
 * strip, row segment) items and one finalize launch; each scenario with its
 * own CFL iteration length and forcing), with continuous admission.
 *
 * A request is queued on submit with a host copy of its inputs.  Every
 * sw2d_batch_step() admits queued requests (first fit, in arrival order)
 * while the HBM budget and the running-slot limit allow, advances all
 * running scenarios by a chunk of iterations (replayed from a captured CUDA
 * graph), and retires the ones that reached their end time: their final
 * depth and discharges are copied to host memory and their device memory is
 * released for the next admissions.  Running state stays on the device
 * between steps.
 *
 * The reference runs one raster per process with no batching (SW2D-EFDC.cu
 * main loop over db/dir.txt cases, :3733-3738, one after the other).
 */
#include "sw2d.h"
#include "sw2d_batch.h"
#include "sw2d_engine.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace {

thread_local std::string g_berr;

int bfail(int code, const std::string& m) {
    g_berr = m;
    return code;
}

struct Request {
    int64_t id = 0;
    int status = SW2D_REQ_QUEUED;
    sw2d_scenario desc{};
    std::vector<double> dem, depth, mtab, rain;
    std::vector<uint8_t> mcls;
    std::vector<float> rainw;
    size_t bytes = 0;
    int engine_index = -1;
    /* results */
    std::vector<double> r_depth, r_qx, r_qy;
    sw2d_ledger ledger{};
    long long iterations = 0;
    double cell_updates = 0;
};

} // namespace

struct sw2d_batch {
    int device = 0;
    double budget = 0;
    int max_running = 0;
    std::unique_ptr<sw2d::Engine32> eng;
    std::map<int64_t, std::unique_ptr<Request>> reqs;
    std::deque<int64_t> queue;
    std::vector<int64_t> running; /* engine index order */
    int64_t next_id = 1;
    double device_ms = 0;
    double cell_updates = 0;
    long long launches = 0;
    long long tuning_iterations = 0; /* iterations advanced by sw2d_batch_tune */
};

static sw2d::ScenarioInput to_input(const Request& r) {
    sw2d::ScenarioInput in;
    const sw2d_scenario& d = r.desc;
    in.rows = d.rows;
    in.cols = d.cols;
    in.dx = d.dx;
    in.dy = d.dy;
    in.nodata = d.nodata;
    in.th = d.th;
    in.g = d.g;
    in.manning = d.manning;
    in.dt_mode = d.dt_mode;
    in.series_mode = d.series_mode;
    in.outflow_south = d.outflow == SW2D_OUTFLOW_SOUTH;
    in.dt = d.dt;
    in.cfl = d.cfl;
    in.dt_max = d.dt_max;
    in.t0 = d.t0;
    in.t_end = d.t_end;
    in.frac_int = d.frac_int;
    in.frac_inf = d.frac_inf;
    in.frac_lwl = d.frac_lwl;
    in.ev_wl_min = d.ev_wl_min;
    in.dem = r.dem.data();
    in.depth = r.depth.empty() ? nullptr : r.depth.data();
    if (!r.mcls.empty()) {
        in.mclass = r.mcls.data();
        in.mtable = r.mtab.data();
        in.ntable = (int)r.mtab.size();
    }
    in.rain = r.rain.data();
    in.nrain = (int)r.rain.size();
    in.dtrain = d.dtrain;
    if (!r.rainw.empty()) in.rain_weight = r.rainw.data();
    in.outlet_cap = d.outlet_capacity;
    return in;
}

/* the ledger of the scenario at engine index k, from its device clock and
 * a volume measure of its current state */
static int read_ledger(sw2d_batch* b, size_t k, sw2d_ledger* out, sw2d::Clock32* clock_out) {
    std::string err;
    sw2d::Clock32 c;
    double vol = 0, smax = 0;
    int rc;
    if ((rc = b->eng->get_clock((int)k, &c, &err))) return bfail(rc, err);
    if ((rc = b->eng->get_volume((int)k, &vol, &smax, &err))) return bfail(rc, err);
    sw2d_ledger& L = *out;
    L.time = c.t;
    L.iterations = (double)c.iters;
    L.volume = vol;
    L.volume0 = c.volume0;
    L.rain_in = c.rain_in;
    L.source_in = c.source_in;
    L.evap_out = c.evap_out;
    L.outflow = c.outflow;
    L.clamp_gain = c.clamp_gain;
    L.q_out = c.q_out;
    L.s_max = c.s_max;
    L.dt_last = c.dt2;
    const double inflow = L.rain_in + L.source_in;
    L.balance_error = (L.volume - L.volume0 - L.rain_in - L.source_in + L.evap_out + L.outflow) /
                      std::max(std::fabs(inflow), 1e-300);
    if (clock_out) *clock_out = c;
    return SW2D_OK;
}

static int retire(sw2d_batch* b, size_t k) {
    const int64_t id = b->running[k];
    Request& r = *b->reqs[id];
    std::string err;
    const size_t n = (size_t)r.desc.rows * r.desc.cols;
    r.r_depth.resize(n);
    r.r_qx.resize((size_t)(r.desc.rows + 1) * r.desc.cols);
    r.r_qy.resize((size_t)r.desc.rows * (r.desc.cols + 1));
    int rc = b->eng->get_state((int)k, r.r_depth.data(), r.r_qx.data(), r.r_qy.data(), &err);
    if (rc) return bfail(rc, err);
    sw2d::Clock32 c;
    if ((rc = read_ledger(b, k, &r.ledger, &c))) return rc;
    r.iterations = c.iters;
    r.status = (c.status & 3) ? SW2D_REQ_FAILED : SW2D_REQ_DONE;
    b->eng->remove((int)k);
    b->running.erase(b->running.begin() + k);
    r.engine_index = -1;
    /* inputs are no longer needed */
    std::vector<double>().swap(r.dem);
    std::vector<double>().swap(r.depth);
    std::vector<uint8_t>().swap(r.mcls);
    std::vector<float>().swap(r.rainw);
    return SW2D_OK;
}

extern "C" {

const char* sw2d_batch_last_error(void) { return g_berr.c_str(); }

int sw2d_batch_create(int device, double hbm_budget_bytes, int max_running, sw2d_batch** out) {
    if (!out || max_running < 0 || hbm_budget_bytes < 0) return bfail(SW2D_ERR_INVALID, "invalid argument");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return bfail(SW2D_ERR_NODEVICE, "no CUDA device");
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess || prop.major != 10 || prop.minor != 3)
        return bfail(SW2D_ERR_NODEVICE, "this library is built for sm_103a (GB300) only");
    auto b = std::make_unique<sw2d_batch>();
    b->device = device;
    b->budget = hbm_budget_bytes;
    b->max_running = max_running;
    b->eng.reset(new sw2d::Engine32(device));
    std::string err;
    int rc = b->eng->init(&err);
    if (rc) return bfail(rc, err);
    *out = b.release();
    return SW2D_OK;
}

int sw2d_batch_destroy(sw2d_batch* b) {
    delete b;
    return SW2D_OK;
}

int sw2d_batch_submit(sw2d_batch* b, const sw2d_scenario* s, int64_t* id_out) {
    if (!b || !s || !s->dem) return bfail(SW2D_ERR_INVALID, "null argument");
    if (s->rows < 2 || s->cols < 2 || !(s->dx > 0) || !(s->dy > 0) || !(s->th > 0))
        return bfail(SW2D_ERR_INVALID, "scenario geometry");
    if ((long long)s->rows * s->cols > (1LL << 30)) return bfail(SW2D_ERR_INVALID, "raster too large");
    if (s->dt_mode != SW2D_DT_FIXED && s->dt_mode != SW2D_DT_CFL) return bfail(SW2D_ERR_INVALID, "dt_mode");
    if (s->series_mode < 0 || s->series_mode > 2) return bfail(SW2D_ERR_INVALID, "series_mode");
    if (s->outlet_capacity < 0) return bfail(SW2D_ERR_INVALID, "outlet_capacity");
    if (s->manning_class && (!s->manning_table || s->ntable <= 0 || s->ntable > 64))
        return bfail(SW2D_ERR_INVALID, "Manning table must have 1..64 entries");
    if ((s->nrain > 0 && !s->rain_mm) || s->nrain < 0 || !(s->dtrain > 0))
        return bfail(SW2D_ERR_INVALID, "rain series");
    if (s->dt_mode == SW2D_DT_CFL && (!(s->cfl > 0) || !(s->dt_max > 0)))
        return bfail(SW2D_ERR_INVALID, "cfl and dt_max must be > 0");
    if (s->dt_mode == SW2D_DT_FIXED && !(s->dt > 0)) return bfail(SW2D_ERR_INVALID, "dt must be > 0");
    const size_t need = sw2d::Engine32::scenario_bytes(s->rows, s->cols, s->rain_weight != nullptr,
                                                       s->outlet_capacity);
    if (b->budget > 0 && (double)need > b->budget)
        return bfail(SW2D_ERR_BUDGET, "scenario larger than the whole HBM budget");
    auto r = std::make_unique<Request>();
    r->id = b->next_id++;
    r->desc = *s;
    const size_t n = (size_t)s->rows * s->cols;
    r->dem.assign(s->dem, s->dem + n);
    if (s->depth) r->depth.assign(s->depth, s->depth + n);
    if (s->manning_class) {
        r->mcls.assign(s->manning_class, s->manning_class + n);
        r->mtab.assign(s->manning_table, s->manning_table + s->ntable);
        for (uint8_t c : r->mcls)
            if (c >= s->ntable) return bfail(SW2D_ERR_INVALID, "Manning class out of table range");
    }
    if (s->nrain > 0) r->rain.assign(s->rain_mm, s->rain_mm + s->nrain);
    else r->rain.assign(1, 0.0);
    if (s->rain_weight) r->rainw.assign(s->rain_weight, s->rain_weight + n);
    r->desc.dem = nullptr;
    r->desc.depth = nullptr;
    r->desc.manning_class = nullptr;
    r->desc.manning_table = nullptr;
    r->desc.rain_mm = nullptr;
    r->desc.rain_weight = nullptr;
    r->bytes = need;
    const int64_t id = r->id;
    b->reqs[id] = std::move(r);
    b->queue.push_back(id);
    if (id_out) *id_out = id;
    return SW2D_OK;
}

/* admit queued requests: first fit in arrival order */
static void admit(sw2d_batch* b) {
    std::string err;
    size_t in_use = b->eng->bytes_in_use();
    for (auto it = b->queue.begin(); it != b->queue.end();) {
        if (b->max_running > 0 && (int)b->running.size() >= b->max_running) break;
        Request& r = *b->reqs[*it];
        if (b->budget > 0 && (double)(in_use + r.bytes) > b->budget) {
            ++it;
            continue;
        }
        int idx = -1;
        int rc = b->eng->add(to_input(r), r.id, &err, &idx);
        if (rc == SW2D_ERR_NOMEM) { /* the device is fuller than the budget says: wait */
            ++it;
            break;
        }
        if (rc) {
            r.status = SW2D_REQ_FAILED;
            it = b->queue.erase(it);
            continue;
        }
        r.status = SW2D_REQ_RUNNING;
        r.engine_index = idx;
        b->running.push_back(r.id);
        in_use += r.bytes;
        it = b->queue.erase(it);
    }
}

int sw2d_batch_step(sw2d_batch* b, int iterations, int* n_running_out, int* n_queued_out) {
    sw2d::NvtxRange r("sw2d_batch_step");
    if (!b || iterations < 0) return bfail(SW2D_ERR_INVALID, "invalid argument");
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(SW2D_ERR_CUDA, "cudaSetDevice");
    std::string err;
    admit(b);
    if (!b->running.empty() && iterations > 0) {
        double cells = 0;
        std::vector<sw2d::Clock32> before(b->running.size());
        for (size_t k = 0; k < b->running.size(); k++) {
            int rc = b->eng->get_clock((int)k, &before[k], &err);
            if (rc) return bfail(rc, err);
        }
        int rc = b->eng->run(iterations, &err);
        if (rc) return bfail(rc, err);
        b->device_ms += b->eng->last_ms();
        b->launches += (long long)((iterations + sw2d::Engine32::kChunk - 1) / sw2d::Engine32::kChunk) *
                       b->eng->launches_per_chunk();
        /* retire finished scenarios (highest index first keeps indices valid) */
        for (size_t k = b->running.size(); k-- > 0;) {
            sw2d::Clock32 c;
            if ((rc = b->eng->get_clock((int)k, &c, &err))) return bfail(rc, err);
            Request& r = *b->reqs[b->running[k]];
            const double cu = (double)(c.iters - before[k].iters) * r.desc.rows * r.desc.cols;
            r.cell_updates += cu;
            cells += cu;
            if (c.done || (c.status & 3)) {
                if ((rc = retire(b, k))) return rc;
            }
        }
        b->cell_updates += cells;
    }
    if (n_running_out) *n_running_out = (int)b->running.size();
    if (n_queued_out) *n_queued_out = (int)b->queue.size();
    return SW2D_OK;
}

int sw2d_batch_poll(sw2d_batch* b, int64_t id, int* status, sw2d_ledger* ledger) {
    if (!b) return bfail(SW2D_ERR_INVALID, "null batch");
    auto it = b->reqs.find(id);
    if (it == b->reqs.end()) return bfail(SW2D_ERR_NOT_FOUND, "unknown request id");
    Request& r = *it->second;
    if (status) *status = r.status;
    if (ledger) {
        if (r.status == SW2D_REQ_RUNNING) {
            /* a running request's ledger as of now, read from the device */
            for (size_t k = 0; k < b->running.size(); k++)
                if (b->running[k] == id) return read_ledger(b, k, ledger, nullptr);
        }
        *ledger = r.ledger;
    }
    return SW2D_OK;
}

int sw2d_batch_result(sw2d_batch* b, int64_t id, double* depth, double* qx, double* qy) {
    if (!b) return bfail(SW2D_ERR_INVALID, "null batch");
    auto it = b->reqs.find(id);
    if (it == b->reqs.end()) return bfail(SW2D_ERR_NOT_FOUND, "unknown request id");
    Request& r = *it->second;
    if (r.status != SW2D_REQ_DONE) return bfail(SW2D_ERR_STATE, "request not finished");
    if (depth) std::memcpy(depth, r.r_depth.data(), r.r_depth.size() * sizeof(double));
    if (qx) std::memcpy(qx, r.r_qx.data(), r.r_qx.size() * sizeof(double));
    if (qy) std::memcpy(qy, r.r_qy.data(), r.r_qy.size() * sizeof(double));
    return SW2D_OK;
}

int sw2d_batch_release(sw2d_batch* b, int64_t id) {
    if (!b) return bfail(SW2D_ERR_INVALID, "null batch");
    auto it = b->reqs.find(id);
    if (it == b->reqs.end()) return bfail(SW2D_ERR_NOT_FOUND, "unknown request id");
    if (it->second->status == SW2D_REQ_RUNNING) {
        for (size_t k = 0; k < b->running.size(); k++)
            if (b->running[k] == id) {
                b->eng->remove((int)k);
                b->running.erase(b->running.begin() + k);
                break;
            }
    }
    for (auto q = b->queue.begin(); q != b->queue.end(); ++q)
        if (*q == id) {
            b->queue.erase(q);
            break;
        }
    b->reqs.erase(it);
    return SW2D_OK;
}

int sw2d_batch_tune(sw2d_batch* b, int max_iterations, int* iterations_out) {
    sw2d::NvtxRange r("sw2d_batch_tune");
    if (!b || max_iterations < 0) return bfail(SW2D_ERR_INVALID, "invalid argument");
    if (cudaSetDevice(b->device) != cudaSuccess) return bfail(SW2D_ERR_CUDA, "cudaSetDevice");
    std::string err;
    admit(b);
    long long done = 0;
    if (!b->running.empty()) {
        int rc = b->eng->tune_now(max_iterations, &err, &done);
        if (rc) return bfail(rc, err);
        for (size_t k = b->running.size(); k-- > 0;) {
            sw2d::Clock32 c;
            if ((rc = b->eng->get_clock((int)k, &c, &err))) return bfail(rc, err);
            if (c.done || (c.status & 3)) {
                if ((rc = retire(b, k))) return rc;
            }
        }
    }
    b->tuning_iterations += done;
    if (iterations_out) *iterations_out = (int)done;
    return SW2D_OK;
}

int sw2d_batch_set_rows_per_item(sw2d_batch* b, int rows) {
    if (!b) return bfail(SW2D_ERR_INVALID, "null batch");
    if (rows != 0 && (rows < 16 || rows > sw2d::M_MAXSEG || rows % 4 != 0))
        return bfail(SW2D_ERR_INVALID, "rows per work item: 0, or a multiple of 4 in 16..512");
    b->eng->set_segment_rows(rows);
    return SW2D_OK;
}

int sw2d_batch_get_stats(sw2d_batch* b, sw2d_batch_stats* out) {
    if (!b || !out) return bfail(SW2D_ERR_INVALID, "null argument");
    out->running = (int)b->running.size();
    out->queued = (int)b->queue.size();
    out->bytes_in_use = (double)b->eng->bytes_in_use();
    out->device_ms = b->device_ms;
    out->cell_updates = b->cell_updates;
    out->launches = (double)b->launches;
    out->work_items = b->eng->nwork();
    out->rows_per_item = b->eng->segment_rows();
    out->tuning_ms = b->eng->tuning_ms();
    out->ctas_per_sm = b->eng->ctas_per_sm();
    out->tunings = b->eng->tunings();
    out->tuning_iterations = (double)b->tuning_iterations;
    return SW2D_OK;
}

} /* extern "C" */
