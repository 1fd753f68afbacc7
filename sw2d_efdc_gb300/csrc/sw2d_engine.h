/* Host engine of the FP32 precision form: owns the scenarios that one
 * persistent launch per feature class advances together, a chunk of
 * iterations at a time (one scenario for a single raster, many for the
 * batched and served forms), and the autotuner that chooses the work split
 * (rows per work item, CTAs per SM) per size bucket. */
#ifndef SW2D_ENGINE_H
#define SW2D_ENGINE_H

#include "sw2d.h"
#include "sw2d_fp32.h"

#include <nvtx3/nvToolsExt.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace sw2d {

/* A named range on the NVTX timeline around a host call (free when no
 * profiler is attached). */
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct ScenarioInput {
    int rows = 0, cols = 0;
    double dx = 1, dy = 1, nodata = -9999.0, th = 1e-4, g = 9.80, manning = 0.03;
    int dt_mode = 1, series_mode = 2, outflow_south = 0;
    double dt = 0.04, cfl = 0.7, dt_max = 2.0, t0 = 0.0, t_end = 0.0;
    double frac_int = 0, frac_inf = 0, frac_lwl = 0, ev_wl_min = 0.05;
    const double* dem = nullptr;        /* rows*cols */
    const double* depth = nullptr;      /* rows*cols or NULL (dry) */
    const uint8_t* mclass = nullptr;    /* rows*cols or NULL */
    const double* mtable = nullptr;
    int ntable = 0;
    const double* rain = nullptr;       /* mm per dtrain */
    int nrain = 0;
    double dtrain = 3600.0;
    const float* rain_weight = nullptr; /* rows*cols or NULL */
    const double* evap = nullptr;       /* evaporation, mm per dtrain, or NULL */
    int nevap = 0;
    int nsrc = 0;                       /* point sources (at most T32_MAXSRC) */
    const int* src_cells = nullptr;     /* nsrc raster ids (row*cols + col) */
    const double* src_q = nullptr;      /* nq rows of nsrc discharges, m3/s */
    int nq = 0;
    double dtoq = 3600.0;
    int outlet_cap = 0;
};

struct Scenario32 {
    Scn32 d{};                 /* host copy of the device descriptor */
    int R = 0, C = 0, P = 0, NR = 0;
    size_t bytes = 0;          /* device bytes held */
    std::vector<void*> allocs;
    double t_end_default = 0.0;
    long long id = -1;
    bool finished = false;
};

class Engine32 {
  public:
    explicit Engine32(int device);
    ~Engine32();
    int init(std::string* err);
    /* device bytes a scenario of this size needs */
    static size_t scenario_bytes(int rows, int cols, bool rain_field, int outlet_cap);
    int add(const ScenarioInput& in, long long id, std::string* err, int* index_out);
    int remove(int index);
    int count() const { return (int)scn_.size(); }
    Scenario32& at(int i) { return *scn_[i]; }
    /* set every scenario's t_end (or one) and recompute first slots */
    int set_t_end(int index, double t_end, std::string* err);
    /* run n iterations of every scenario (finished ones idle) */
    int run(long long n, std::string* err);
    /* state of one scenario, reference orientation */
    int get_state(int index, double* depth, double* qx, double* qy, std::string* err);
    int get_clock(int index, Clock32* out, std::string* err);
    int get_volume(int index, double* vol, double* smax, std::string* err);
    int get_outlet(int index, double* t, double* q, int cap, int* count, std::string* err);
    /* the scenario's device state (clock, then depth, x and y discharges and
     * the Kahan compensation, whole padded arrays) to / from a host buffer of
     * snapshot_bytes(index) bytes */
    /* failure test: the scenario's work items issue no staged loads, so the
     * kernel's bounded wait gives up and sets the timeout status bit */
    void set_stall_staging(int index, bool on) {
        scn_[index]->d.stall_staging = on ? 1 : 0;
        dirty_ = true;
    }
    size_t snapshot_bytes(int index) const;
    int snapshot(int index, void* buf, std::string* err);
    int restore(int index, const void* buf, std::string* err);
    cudaStream_t stream() const { return stream_; }
    /* the device descriptor of scenario i (valid after the work list is built) */
    const Scn32* device_scenario(int i) {
        std::string e;
        return rebuild(&e) == SW2D_OK ? d_scn_ + i : nullptr;
    }
    size_t bytes_in_use() const;
    double last_ms() const { return last_ms_; }
    long long last_iters() const { return last_iters_; }
    int nwork() const { return (int)work_.size(); }
    /* kernel launches of one chunk of iterations: one persistent launch per
     * feature class present */
    int launches_per_chunk() const {
        int n = 0;
        for (int k = 0; k < T32_NCLASS; k++) n += class_n_[k] > 0 ? 1 : 0;
        return n;
    }
    /* iterations one chunk (one persistent launch per class) advances */
    static constexpr int kChunk = 32;
    int sync(std::string* err);
    /* rows per work item (16..512; 0 = chosen by the autotuner).  The
     * results do not depend on it: the bed's datum tiles are fixed. */
    void set_segment_rows(int rows) {
        seg_fixed_ = rows;
        if (rows > 0 && rows != seg_) {
            seg_ = rows;
            dirty_ = true;
        }
        tuned_.clear();
        bucket_ = -1;
    }
    int segment_rows() const { return seg_; }
    /* CTAs per SM of the persistent launches (the autotuner's second
     * choice; 0 = every CTA the SM holds) */
    int ctas_per_sm() const { return cps_; }
    /* host milliseconds the autotuner spent timing candidates (the
     * iterations it timed were real ones: they advanced the scenarios) */
    double tuning_ms() const { return tuning_ms_; }
    int tunings() const { return tunings_; }
    /* the autotuner now, for the work set's size bucket, advancing the
     * scenarios by at most `budget` iterations (*advanced of them; 0 when
     * the bucket is tuned already or the budget holds too few) */
    int tune_now(long long budget, std::string* err, long long* advanced);

  private:
    int rebuild(std::string* err);
    int build_graph(std::string* err);
    int launch(int niter, std::string* err);
    /* the autotuner: times each candidate pair (rows per item, CTAs per
     * SM) on the scenarios' own iterations -- one untimed, then up to a
     * chunk's worth in one persistent launch, as the chunks run -- and keeps
     * the fastest, cached per size bucket (log2 of the work set's cells).
     * Advances at most `budget` iterations and returns how many. */
    int tune(long long budget, std::string* err, long long* advanced);
    int grid_of(int k, int niter) const;
    int device_;
    int nsm_ = 0;
    int bps_[T32_NCLASS] = {};  /* CTAs per SM of each class's persistent kernel */
    cudaStream_t stream_ = nullptr;
    std::vector<std::unique_ptr<Scenario32>> scn_;
    std::vector<int4> work_;
    int class_first_[T32_NCLASS] = {}, class_n_[T32_NCLASS] = {}; /* work ranges per feature class */
    Scn32* d_scn_ = nullptr;
    size_t d_scn_cap_ = 0;
    int4* d_work_ = nullptr;
    size_t d_work_cap_ = 0;
    Part32* d_part_ = nullptr;
    void* d_ctl_ = nullptr;    /* persistent-launch control block, fp32_ctl_bytes */
    size_t d_ctl_cap_ = 0;
    double* d_tmp_ = nullptr;
    bool dirty_ = true;
    cudaGraphExec_t graph_ = nullptr;
    bool graph_failed_ = false; /* capture of the cooperative launch refused: launch directly */
    cudaEvent_t ev_a_ = nullptr, ev_b_ = nullptr, ev_t0_ = nullptr, ev_t1_ = nullptr;
    double last_ms_ = 0.0;
    long long last_iters_ = 0;
    int seg_ = 128;            /* rows per work item in use */
    int seg_fixed_ = 0;        /* set by set_segment_rows or SW2D_SEGMENT_ROWS */
    int cps_ = 0;              /* CTAs per SM in use (0: all that fit) */
    int bucket_ = -1;          /* size bucket the setting in use was chosen for */
    std::map<int, std::pair<int, int>> tuned_; /* size bucket -> (rows per item, CTAs per SM) */
    double tuning_ms_ = 0.0;
    int tunings_ = 0;
    void* pin_ = nullptr;      /* pinned staging of state downloads */
    size_t pin_bytes_ = 0;
};

} // namespace sw2d
#endif
