/* sw2d_cli -- the reference's case driver on this library.
 *
 * The reference's only entry point is main() (SW2D-EFDC.cu:3682-5166): it
 * reads db/dir.txt, then for each case db/<case>/setup.dat and the
 * SW2D/input files, runs the explicit step with a fixed dt and writes
 * SW2D/output/Results_<t>.vtk, WaterLevel.txt and TimeSimu_<t>.txt; a
 * coupled case (setup.dat "3D HYDRODYNAMIC MODEL" = 1) also smooths the DEM
 * along the lake edge and writes the EFDC hand-off decks.  This program reads
 * the same tree and writes the same files through the C ABI (include/sw2d.h),
 * FP64 by default, so the outputs are the reference's.
 *
 *   sw2d_cli [--root DIR] [--check] [--fp32] [--device N] [--quiet]
 *
 *   --root DIR  directory holding db/ (default: the working directory, as the
 *               reference reads "db/dir.txt")
 *   --check     read and validate every input, print a JSON summary of each
 *               case (sizes, times, output schedule, sources, outlets) and
 *               run nothing: needs no GPU
 *   --fp32      run the FP32 form of the step (faster; not bit-identical)
 *   --device N  CUDA device ordinal (default 0)
 *   --quiet     no progress lines
 *
 * Coupled cases: the SW2D side of the hand-off is written (EFDC/input/EFDC.INP
 * from the template with cards C22-C26 for the boundary faces, QSER.INP,
 * and DSER/TSER/SSER.INP when dye / temperature / salinity are on).  The
 * EFDC-MPI run itself, the Gorp domain decomposition, Grid_efdc and the
 * WSER/ASER/SHOW/DYE/SALT/TEMP decks belong to the lake model and are not
 * produced here.
 *
 * Exit status: 0 when every case ran; 1 when an input is missing or
 * malformed (the message names it; the reference prints "unknown file - X"
 * and stops in the same places); 2 when a library call fails.
 */
#include "sw2d.h"

#include <cuda_runtime.h>

#include <sys/stat.h>
#include <sys/types.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <new>
#include <string>
#include <thread>
#include <vector>

namespace {

/* ---------------------------------------------------------------- errors */

struct InputError {
    std::string msg;
};
struct LibError {
    std::string msg;
};

[[noreturn]] void input_error(const std::string& msg) { throw InputError{msg}; }

void check(int rc, const char* what) {
    if (rc != SW2D_OK) throw LibError{std::string(what) + ": " + sw2d_status_string(rc) + ": " + sw2d_last_error()};
}

/* ------------------------------------------------------------ text input */

bool is_ws(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

bool read_file(const std::string& path, std::string* out) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::string s;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, n);
    std::fclose(f);
    out->swap(s);
    return true;
}

/* A whole input file read the way the reference's fscanf calls read it:
 * white space (including CR) separates items, numbers are read by strtod /
 * strtol from the current position. */
class Reader {
public:
    Reader(const std::string& path, const std::string& shown) : name_(shown) {
        if (!read_file(path, &s_)) input_error("unknown file - " + shown);
    }
    const std::string& name() const { return name_; }
    /* lines as the reference counts them: the number of '\n' bytes */
    long newlines() const { return (long)std::count(s_.begin(), s_.end(), '\n'); }
    void skip_ws() {
        while (p_ < s_.size() && is_ws(s_[p_])) p_++;
    }
    /* white space and '#' ... '#' comment blocks (setup.dat's labels) */
    void skip_comments() {
        for (;;) {
            skip_ws();
            if (p_ < s_.size() && s_[p_] == '#') {
                const size_t e = s_.find('#', p_ + 1);
                p_ = (e == std::string::npos) ? s_.size() : e + 1;
                continue;
            }
            return;
        }
    }
    bool token(std::string* t) {
        skip_ws();
        if (p_ >= s_.size()) return false;
        const size_t b = p_;
        while (p_ < s_.size() && !is_ws(s_[p_])) p_++;
        t->assign(s_, b, p_ - b);
        return true;
    }
    /* the keyword of a header line ("ncols", "n_out", ...), matched like a
     * literal of an fscanf format (case-insensitive here) */
    void keyword(const char* k) {
        skip_ws();
        const size_t n = std::strlen(k);
        if (s_.size() - p_ < n || strncasecmp(s_.c_str() + p_, k, n) != 0)
            input_error(name_ + ": expected '" + k + "'" + near());
        p_ += n;
    }
    bool number(double* v) {
        skip_ws();
        if (p_ >= s_.size()) return false;
        const char* b = s_.c_str() + p_;
        char* e = nullptr;
        const double x = std::strtod(b, &e);
        if (e == b) return false;
        p_ += (size_t)(e - b);
        *v = x;
        return true;
    }
    double need_number(const char* what) {
        double v;
        if (!number(&v)) input_error(name_ + ": expected a number for " + what + near());
        return v;
    }
    bool integer(long* v) {
        skip_ws();
        if (p_ >= s_.size()) return false;
        const char* b = s_.c_str() + p_;
        char* e = nullptr;
        const long x = std::strtol(b, &e, 10);
        if (e == b) return false;
        p_ += (size_t)(e - b);
        *v = x;
        return true;
    }
    int need_int(const char* what) {
        long v;
        if (!integer(&v) || v < INT32_MIN || v > INT32_MAX) input_error(name_ + ": expected an integer for " + what + near());
        if (p_ < s_.size() && !is_ws(s_[p_]) && s_[p_] != '#')
            input_error(name_ + ": expected an integer for " + what + near());
        return (int)v;
    }
    /* read up to n numbers; returns how many were present */
    size_t numbers(double* out, size_t n) {
        size_t k = 0;
        while (k < n && number(&out[k])) k++;
        return k;
    }

private:
    std::string near() const {
        const size_t b = std::min(p_, s_.size());
        std::string t = s_.substr(b, 24);
        for (char& c : t)
            if (c == '\n' || c == '\r') c = ' ';
        return t.empty() ? " (end of file)" : " near '" + t + "'";
    }
    std::string s_;
    std::string name_;
    size_t p_ = 0;
};

/* ------------------------------------------------------------- the case */

/* setup.dat section 2 (read only when the 3-D model is on), in file order;
 * the names are the reference's variables (SW2D-EFDC.cu:3814-3958). */
struct Field2 {
    const char* name;
    bool integer;
};
const Field2 kSection2[] = {
    {"efdc_basetime", false}, {"TBEGIN", false}, {"NTSPTC", true}, {"nlayers", true}, {"ZBRADJ", false},
    {"ZBRCVRT", false}, {"HMIN", false}, {"HADJ", false}, {"HCVRT", false}, {"HDRY", false}, {"HWET", false},
    {"BELADJ", false}, {"BELCVRT", false}, {"NWSER", true}, {"NASER", true}, {"IASWRAD", true}, {"REVC", false},
    {"RCHC", false}, {"SWRATNF", false}, {"SWRATNS", false}, {"FSWRATF", false}, {"DABEDT", false},
    {"TBEDIT", false}, {"HTBED1", false}, {"HTBED2", false}, {"ISPPH", true}, {"NPPPH", true}, {"ISRPPH", true},
    {"IPPHXY", true}, {"ISVPH", true}, {"NPVPH", true}, {"ISRVPH", true}, {"IVPHXY", true}, {"NTSSSS", true},
    {"MTSP", true}, {"MTSC", true}, {"MTSA", true}, {"MTSUE", true}, {"MTSUT", true}, {"MTSU", true},
    {"NSTYPE", true}, {"NSHOWR", true}, {"ISHOWC", true}, {"JSHOWC", true}, {"NSHFREQ", true}, {"ZSSMIN", true},
    {"ZSSMAX", true}, {"SSALMAX", true}, {"N_processors", true}, {"Lorp_type", true}, {"dye_on", true},
    {"temp_on", true}, {"salt_on", true}, {"DYE_INIT", false}, {"SALT_INIT", false}, {"TEMP_BOT", false},
    {"TEMP_SURF", false}, {"DYE_IN", false}, {"SALT_IN", false},
};
constexpr int kNSection2 = sizeof kSection2 / sizeof *kSection2;

struct Grid {
    int cols = 0, rows = 0;
    double xll = 0, yll = 0, cellsize = 0, nodata = 0;
};

struct Case {
    std::string name, dir;
    /* setup.dat section 1 (SW2D-EFDC.cu:3763-3808) */
    double t0[4] = {}, t1[4] = {};
    double dt = 0, dpout = 0, dkout = 0, dtoq = 0;
    int evaporation_on = 0;
    double ev_wl_min = 0, frac_int = 0, frac_inf = 0, frac_lwl = 0, manning = 0;
    int out_vx = 0, out_vy = 0, out_elev = 0, out_depth = 0, out_outlet = 0, efdc = 0;
    double s2[kNSection2] = {};
    /* inputs */
    Grid grid;
    std::vector<double> dem, h0;
    std::vector<int> src_cells;
    std::vector<double> src_q; /* nq rows of nsrc */
    int nq = 0;
    double dtrain = 0;
    std::vector<double> rain, temp, rad, evap;
    double albedo = 0;
    std::vector<long long> outlet_cell; /* raster id each outlet's depth is read at; <0 = outside */
    int n_out = 0;
    std::vector<int> mask;
    /* times (SW2D-EFDC.cu:4230-4234) and step counts (:4187-4188) */
    double time0 = 0, timmax = 0;
    long lpout = 0, lkout = 0;

    double s2v(const char* n) const {
        for (int k = 0; k < kNSection2; k++)
            if (std::strcmp(kSection2[k].name, n) == 0) return s2[k];
        return 0;
    }
    size_t cells() const { return (size_t)grid.rows * grid.cols; }
};

std::string join(const std::string& a, const std::string& b) { return a.empty() ? b : a + "/" + b; }

void read_grid_header(Reader& r, Grid* g) {
    r.keyword("ncols");
    g->cols = r.need_int("ncols");
    r.keyword("nrows");
    g->rows = r.need_int("nrows");
    r.keyword("xllcorner");
    g->xll = r.need_number("xllcorner");
    r.keyword("yllcorner");
    g->yll = r.need_number("yllcorner");
    r.keyword("cellsize");
    g->cellsize = r.need_number("cellsize");
    r.keyword("NODATA_value");
    g->nodata = r.need_number("NODATA_value");
    if (g->cols < 1 || g->rows < 1) input_error(r.name() + ": ncols and nrows must be >= 1");
    /* the library's limit: rows * cols <= 2^30 cells */
    if ((long long)g->cols * g->rows > (1LL << 30)) input_error(r.name() + ": more than 2^30 cells");
    if (!(g->cellsize > 0) || !std::isfinite(g->cellsize)) input_error(r.name() + ": cellsize must be > 0");
}

void read_setup(Case& c) {
    Reader r(join(c.dir, "setup.dat"), "setup.dat");
    auto num = [&](const char* what) {
        r.skip_comments();
        return r.need_number(what);
    };
    auto integ = [&](const char* what) {
        r.skip_comments();
        return r.need_int(what);
    };
    for (int k = 0; k < 4; k++) c.t0[k] = num("START TIME");
    for (int k = 0; k < 4; k++) c.t1[k] = num("END TIME");
    c.dt = num("TIME STEP");
    c.dpout = num("TIME INTERVAL TO SHOW TIME");
    c.dkout = num("TIME INTERVAL TO WRITE THE RESULTS");
    c.dtoq = num("TEMPORAL RESOLUTION OF FLOW INPUT DATA");
    c.evaporation_on = integ("EVAPORATION IN THE LAKE");
    c.ev_wl_min = num("MINIMUM WATER DEPTH FOR EVAPORATION");
    c.frac_int = num("PERCENTAGE OF WATER LOST BY INTERCEPTION");
    c.frac_inf = num("PERCENTAGE OF WATER LOST BY INFILTRATION");
    c.frac_lwl = num("PERCENTAGE OF WATER LOSS IN THE LAKE");
    c.manning = num("MANNING COEFFICIENT");
    c.out_vx = integ("OUTPUT X VELOCITY");
    c.out_vy = integ("OUTPUT Y VELOCITY");
    c.out_elev = integ("OUTPUT ELEVATIONS");
    c.out_depth = integ("OUTPUT WATER DEPTH");
    c.out_outlet = integ("OUTPUT WATER DEPTH TIME SERIES");
    c.efdc = integ("3D HYDRODYNAMIC MODEL");
    if (c.efdc == 1)
        for (int k = 0; k < kNSection2; k++)
            c.s2[k] = kSection2[k].integer ? (double)integ(kSection2[k].name) : num(kSection2[k].name);
    if (!(c.dt > 0) || !std::isfinite(c.dt)) input_error("setup.dat: TIME STEP must be > 0");
}

/* round(interval / dt) as the reference's integer step counts; an interval
 * that is not a positive number of steps gives 0, one beyond 2^62 steps
 * gives 2^62 (never reached) */
long steps_of(double interval, double dt) {
    const double v = std::round(interval / dt);
    if (!(v >= 1.0)) return 0;
    return v > 4.6e18 ? (1L << 62) : (long)v;
}

constexpr double kMaxIterations = 1e10;
constexpr double kMaxRecords = 1e8;

/* the reference's point-source and outlet cell rule (stream_flow,
 * SW2D-EFDC.cu:540-544; outlets :4990-4993): column round(|x0 - x|),
 * row rows - round(|y0 - y|), raster id row*cols + column + 1 */
long long ref_cell(const Grid& g, double x_cells, double y_cells) {
    const double x0 = g.xll / g.cellsize, y0 = g.yll / g.cellsize;
    const long long col = (long long)std::round(std::fabs(x0 - x_cells));
    const long long row = g.rows - (long long)std::round(std::fabs(y0 - y_cells));
    return row * g.cols + col + 1;
}

void read_inputs(Case& c) {
    const std::string in = join(c.dir, "SW2D/input");
    /* DEM: ESRI ASCII grid with N = rows*cols + cols/2 values (SW2D-EFDC.cu:3983-4003) */
    {
        Reader r(join(in, "dem.dat"), "dem.dat");
        read_grid_header(r, &c.grid);
        c.dem.assign(c.cells(), 0.0);
        const size_t got = r.numbers(c.dem.data(), c.cells());
        if (got < c.cells())
            input_error("dem.dat: " + std::to_string(got) + " values, the grid needs " + std::to_string(c.cells()));
    }
    const Grid& g = c.grid;
    /* point sources (SW2D-EFDC.cu:4008-4026) */
    {
        Reader r(join(in, "coord_source_sink.dat"), "coord_source_sink.dat");
        r.keyword("nst");
        const int nst = r.need_int("nst");
        if (nst < 0) input_error("coord_source_sink.dat: nst < 0");
        for (int k = 0; k < nst; k++) {
            const double x = r.need_number("a source x") / g.cellsize;
            const double y = r.need_number("a source y") / g.cellsize;
            const long long cell = ref_cell(g, x, y);
            if (cell < 0 || cell >= (long long)c.cells())
                input_error("coord_source_sink.dat: source " + std::to_string(k + 1) + " lies outside the grid");
            c.src_cells.push_back((int)cell);
        }
    }
    /* discharges: "flow <unit>" then one row of nst values per line
     * (SW2D-EFDC.cu:4031-4070); the reference reserves one row per line of
     * the file, rows the file does not fill hold zeros here */
    {
        Reader r(join(in, "Q_source_sink.dat"), "Q_source_sink.dat");
        const long rows = r.newlines();
        const size_t nst = c.src_cells.size();
        r.keyword("flow");
        std::string unit;
        r.token(&unit);
        c.nq = (int)std::max(rows, 1L);
        c.src_q.assign((size_t)c.nq * nst, 0.0);
        r.numbers(c.src_q.data(), c.src_q.size());
    }
    /* rain: dtrain, a 4-word header, then "<time> <mm>" rows; the reference
     * reads (lines - 1) rows (SW2D-EFDC.cu:4078-4108) */
    long nrain;
    {
        Reader r(join(in, "rain.dat"), "rain.dat");
        nrain = r.newlines() - 1;
        c.dtrain = r.need_number("dtrain");
        std::string h;
        for (int k = 0; k < 4; k++)
            if (!r.token(&h)) input_error("rain.dat: the header needs 4 words");
        if (nrain < 1) input_error("rain.dat: no rain rows");
        c.rain.assign((size_t)nrain, 0.0);
        for (long k = 0; k < nrain; k++) {
            std::string t;
            if (!r.token(&t) || !r.number(&c.rain[(size_t)k])) break;
        }
        if (!(c.dtrain > 0)) input_error("rain.dat: dtrain must be > 0");
    }
    /* temperature and radiation series, as long as the rain series
     * (SW2D-EFDC.cu:4116-4164); temperature also feeds TSER.INP */
    const bool temp_needed = c.evaporation_on == 1 || (c.efdc == 1 && (int)c.s2v("temp_on") == 1);
    if (temp_needed) {
        Reader t(join(in, "temperatures.dat"), "temperatures.dat");
        std::string h;
        t.token(&h);
        c.temp.assign((size_t)nrain, 0.0);
        t.numbers(c.temp.data(), c.temp.size());
    }
    if (c.evaporation_on == 1) {
        Reader s(join(in, "solar_radiation.dat"), "solar_radiation.dat");
        s.keyword("albedo:");
        c.albedo = s.need_number("albedo");
        std::string h;
        s.token(&h);
        c.rad.assign((size_t)nrain, 0.0);
        s.numbers(c.rad.data(), c.rad.size());
        c.evap.assign((size_t)nrain, 0.0);
        check(sw2d_evaporation_series((int)nrain, c.temp.data(), c.rad.data(), c.albedo, c.dtrain, c.evap.data()),
              "sw2d_evaporation_series");
    }
    /* initial depths, N values (SW2D-EFDC.cu:4170-4181) */
    {
        Reader r(join(in, "initial_condition.dat"), "initial_condition.dat");
        c.h0.assign(c.cells(), 0.0);
        const size_t got = r.numbers(c.h0.data(), c.cells());
        if (got < c.cells())
            input_error("initial_condition.dat: " + std::to_string(got) + " values, the grid needs " +
                        std::to_string(c.cells()));
    }
    /* outlets whose depth goes to WaterLevel.txt (SW2D-EFDC.cu:4195-4215) */
    if (c.out_outlet == 1) {
        Reader r(join(in, "coord_out.dat"), "coord_out.dat");
        r.keyword("n_out");
        c.n_out = r.need_int("n_out");
        if (c.n_out < 0) input_error("coord_out.dat: n_out < 0");
        for (int k = 0; k < c.n_out; k++) {
            const double x = r.need_number("an outlet x") / g.cellsize;
            const double y = r.need_number("an outlet y") / g.cellsize;
            const long long cell = ref_cell(g, x, y) - g.cols; /* km = (outy-1)*cols + outx + 1 */
            c.outlet_cell.push_back(cell >= 0 && cell < (long long)c.cells() ? cell : -1);
        }
    }
    /* lake mask of a coupled run (SW2D-EFDC.cu:4340-4362) */
    if (c.efdc == 1) {
        Reader r(join(in, "mask.dat"), "mask.dat");
        Grid mg;
        read_grid_header(r, &mg);
        if (mg.cols != g.cols || mg.rows != g.rows || mg.xll != g.xll || mg.yll != g.yll ||
            mg.cellsize != g.cellsize || mg.nodata != g.nodata)
            input_error("mask.dat: its header differs from dem.dat's");
        c.mask.assign(c.cells(), 0);
        for (size_t k = 0; k < c.cells(); k++) {
            long v;
            if (!r.integer(&v)) input_error("mask.dat: fewer values than the grid's cells");
            c.mask[k] = (int)v;
        }
        if ((int)c.s2v("nlayers") < 1) input_error("setup.dat: NUMBER OF VERTICAL LAYERS must be >= 1");
        if (!(c.s2v("efdc_basetime") > 0)) input_error("setup.dat: EFDC BASE TIME must be > 0");
    }
    /* times (SW2D-EFDC.cu:4230-4234) and output intervals in steps (:4187-4188) */
    c.time0 = 3600.0 * 24.0 * c.t0[0] + 3600.0 * c.t0[1] + 60.0 * c.t0[2] + c.t0[3];
    c.timmax = 3600.0 * 24.0 * c.t1[0] + 3600.0 * c.t1[1] + 60.0 * c.t1[2] + c.t1[3];
    if (c.t1[0] == 0 && c.t1[1] == 0 && c.t1[2] == 0 && c.t1[3] == 0) c.timmax = (double)(nrain - 1) * c.dtrain;
    c.lpout = steps_of(c.dpout, c.dt);
    c.lkout = steps_of(c.dkout, c.dt);
    if (c.lkout < 1) input_error("setup.dat: TIME INTERVAL TO WRITE THE RESULTS must be at least half a TIME STEP");
    if (!c.src_cells.empty() && !(c.dtoq > 0 && std::isfinite(c.dtoq)))
        input_error("setup.dat: TEMPORAL RESOLUTION OF FLOW INPUT DATA must be > 0 with point sources");
    if (!std::isfinite(c.time0) || !std::isfinite(c.timmax)) input_error("setup.dat: the start and end times must be finite");
    /* the schedule is walked iteration by iteration (the reference's time
     * accumulation); bound the walk and what it keeps */
    const double iters = (c.timmax - c.time0) / (2.0 * c.dt);
    if (iters > kMaxIterations) input_error("setup.dat: the run needs more than 1e10 iterations");
    if (iters > 0 && (2.0 * iters / (double)c.lkout > kMaxRecords ||
                      (c.lpout > 0 && 2.0 * iters / (double)c.lpout > kMaxRecords)))
        input_error("setup.dat: more than 1e8 result or progress records");
}

/* ------------------------------------------------------------ schedule */

/* The reference's loop (SW2D-EFDC.cu:4798-4957): before iteration k the time
 * is printed when mstep % lpout == 0; after it, results are written when
 * mstep % lkout == 0 or k is the first iteration; mstep grows by 2 and the
 * time by dt twice per iteration. */
struct Event {
    long long iteration; /* 1-based iteration after which the output is written */
    long long mstep;
    std::string tempo;   /* the file name's time label */
};

std::string label(double v) {
    char b[64];
    std::snprintf(b, sizeof b, "%g", v); /* an ostream's default format */
    return b;
}

void schedule(const Case& c, std::vector<Event>* ev, std::vector<std::pair<long long, int>>* prints,
              long long* iterations) {
    double time = c.time0;
    long long mstep = 0, out0 = -1, k = 0;
    while (time + c.dt <= c.timmax) {
        out0++;
        if (c.lpout > 0 && mstep % c.lpout == 0) prints->push_back({k + 1, (int)time});
        time = time + c.dt;
        time = time + c.dt;
        mstep += 2;
        k++;
        if (mstep % c.lkout == 0 || out0 == 0)
            ev->push_back({k, mstep, out0 > 0 ? label(std::round((double)mstep * c.dt / c.dkout)) : "0"});
    }
    *iterations = k;
}

/* -------------------------------------------------------------- outputs */

/* lines "%f\n" of v[(rows-1-i)*cols + j], i.e. the raster from its last row
 * up, formatted on all host threads (the bytes of one fprintf per value) */
void write_field(FILE* f, const std::vector<double>& v, int rows, int cols, double sign) {
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const int per = (rows + (int)nt - 1) / (int)nt;
    std::vector<std::string> parts(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; t++)
        th.emplace_back([&, t] {
            std::string& s = parts[t];
            char b[64];
            const int i0 = (int)t * per, i1 = std::min(rows, i0 + per);
            for (int i = i0; i < i1; i++) {
                const double* row = &v[(size_t)(rows - 1 - i) * cols];
                for (int j = 0; j < cols; j++) {
                    const int n = std::snprintf(b, sizeof b, "%f\n", sign < 0 ? -row[j] : row[j]);
                    s.append(b, (size_t)n);
                }
            }
        });
    for (auto& x : th) x.join();
    for (auto& s : parts) std::fwrite(s.data(), 1, s.size(), f);
}

void make_dirs(const std::string& path) {
    std::string cur;
    size_t p = 0;
    while (p != std::string::npos) {
        p = path.find('/', p + 1);
        cur = path.substr(0, p);
        if (!cur.empty()) mkdir(cur.c_str(), 0777);
    }
}

FILE* open_out(const std::string& path) {
    FILE* f = std::fopen(path.c_str(), "w");
    if (!f) input_error("cannot write " + path);
    return f;
}

/* ------------------------------------------------------------------ run */

struct Options {
    std::string root;
    bool check = false, fp32 = false, quiet = false;
    int device = 0;
};

std::string json_str(const std::string& v) {
    std::string o;
    for (unsigned char ch : v) {
        if (ch == '"' || ch == '\\') {
            o += '\\';
            o += (char)ch;
        } else if (ch < 0x20) {
            char b[8];
            std::snprintf(b, sizeof b, "\\u%04x", ch);
            o += b;
        } else {
            o += (char)ch;
        }
    }
    return o;
}

void print_check(const Case& c, const std::vector<Event>& ev, long long iters) {
    std::printf("{\"case\": \"%s\", \"rows\": %d, \"cols\": %d, \"cellsize\": %.17g, \"nodata\": %.17g, "
                "\"xllcorner\": %.17g, \"yllcorner\": %.17g, \"dt\": %.17g, \"time0\": %.17g, \"timmax\": %.17g, "
                "\"lpout\": %ld, \"lkout\": %ld, \"iterations\": %lld, \"manning\": %.17g, "
                "\"fractions\": [%.17g, %.17g, %.17g], \"ev_wl_min\": %.17g, \"evaporation\": %d, "
                "\"dtrain\": %.17g, \"nrain\": %zu, \"rain_total\": %.17g, \"evap_total\": %.17g, "
                "\"dem_total\": %.17g, \"h0_total\": %.17g, \"efdc\": %d",
                json_str(c.name).c_str(), c.grid.rows, c.grid.cols, c.grid.cellsize, c.grid.nodata, c.grid.xll, c.grid.yll,
                c.dt, c.time0, c.timmax, c.lpout, c.lkout, iters, c.manning, c.frac_int, c.frac_inf, c.frac_lwl,
                c.ev_wl_min, c.evaporation_on, c.dtrain, c.rain.size(), [&] {
                    double s = 0;
                    for (double v : c.rain) s += v;
                    return s;
                }(),
                [&] {
                    double s = 0;
                    for (double v : c.evap) s += v;
                    return s;
                }(),
                [&] {
                    double s = 0;
                    for (double v : c.dem) s += v;
                    return s;
                }(),
                [&] {
                    double s = 0;
                    for (double v : c.h0) s += v;
                    return s;
                }(),
                c.efdc);
    std::printf(", \"sources\": [");
    for (size_t k = 0; k < c.src_cells.size(); k++) std::printf("%s%d", k ? ", " : "", c.src_cells[k]);
    std::printf("], \"nq\": %d, \"q_total\": %.17g", c.nq, [&] {
        double s = 0;
        for (double v : c.src_q) s += v;
        return s;
    }());
    std::printf(", \"outlets\": [");
    for (size_t k = 0; k < c.outlet_cell.size(); k++) std::printf("%s%lld", k ? ", " : "", c.outlet_cell[k]);
    std::printf("], \"outputs\": [");
    for (size_t k = 0; k < ev.size(); k++)
        std::printf("%s[%lld, \"%s\"]", k ? ", " : "", ev[k].iteration, ev[k].tempo.c_str());
    std::printf("]");
    if (c.efdc == 1) {
        long lake = 0;
        for (int m : c.mask) lake += m == 1;
        std::printf(", \"lake_cells\": %ld, \"nlayers\": %d, \"efdc_basetime\": %.17g, \"dye_on\": %d, "
                    "\"temp_on\": %d, \"salt_on\": %d",
                    lake, (int)c.s2v("nlayers"), c.s2v("efdc_basetime"), (int)c.s2v("dye_on"),
                    (int)c.s2v("temp_on"), (int)c.s2v("salt_on"));
    }
    std::printf("}\n");
}


/* The coupled run's DEM pre-pass (lake_catchment_smooth, SW2D-EFDC.cu:2766-2827)
 * on the device: the mask and the DEM are copied to the run's GPU, smoothed
 * there by the library's wavefront pass and copied back before the DEM is
 * loaded. */
static void smooth_lake_edges_on_device(int device, int R, int C, const std::vector<int>& mask,
                                        std::vector<double>& dem) {
    const size_t n = (size_t)R * C;
    int* dm = nullptr;
    double* dz = nullptr;
    bool ok = cudaSetDevice(device) == cudaSuccess && cudaMalloc(&dm, n * sizeof(int)) == cudaSuccess &&
              cudaMalloc(&dz, n * sizeof(double)) == cudaSuccess &&
              cudaMemcpy(dm, mask.data(), n * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess &&
              cudaMemcpy(dz, dem.data(), n * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
    if (ok) check(sw2d_lake_catchment_smooth_device(R, C, dm, dz, nullptr), "sw2d_lake_catchment_smooth_device");
    ok = ok && cudaMemcpy(dem.data(), dz, n * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(dm);
    cudaFree(dz);
    if (!ok) {
        std::fprintf(stderr, "sw2d_cli: CUDA error in the lake-edge pre-pass: %s\n", cudaGetErrorString(cudaGetLastError()));
        std::exit(1);
    }
}

void run_case(Case& c, const Options& o) {
    const Grid& g = c.grid;
    const int R = g.rows, C = g.cols;
    const std::string out_dir = join(c.dir, "SW2D/output");
    const std::string efdc_dir = join(c.dir, "EFDC/input");
    std::vector<Event> ev;
    std::vector<std::pair<long long, int>> prints;
    long long iters = 0;
    schedule(c, &ev, &prints, &iters);
    if (o.check) {
        print_check(c, ev, iters);
        return;
    }
    make_dirs(out_dir);
    const bool coupled = c.efdc == 1;
    if (coupled) {
        /* the template deck is copied first (SW2D-EFDC.cu:4271-4281) */
        std::string tpl;
        if (!read_file(join(efdc_dir, "template/EFDC.INP"), &tpl)) input_error("unknown file - EFDC/input/template/EFDC.INP");
        FILE* f = open_out(join(efdc_dir, "EFDC.INP"));
        std::fwrite(tpl.data(), 1, tpl.size(), f);
        std::fclose(f);
        smooth_lake_edges_on_device(o.device, R, C, c.mask, c.dem);
    }
    FILE* wl = open_out(join(out_dir, "WaterLevel.txt"));
    if (c.out_outlet != 1) std::fprintf(wl, "%s\n", "Outlet off");

    sw2d_config cfg;
    sw2d_config_default(&cfg);
    cfg.rows = R;
    cfg.cols = C;
    cfg.precision = o.fp32 ? SW2D_FP32 : SW2D_FP64;
    cfg.dt_mode = SW2D_DT_FIXED;
    cfg.series_mode = SW2D_SERIES_REFERENCE;
    cfg.outflow = SW2D_OUTFLOW_NONE;
    cfg.device = o.device;
    cfg.dx = cfg.dy = g.cellsize;
    cfg.nodata = g.nodata;
    cfg.th = 1.0e-4;
    cfg.g = 9.80;
    cfg.manning = c.manning;
    cfg.dt = c.dt;
    cfg.t0 = c.time0;
    cfg.frac_int = c.frac_int;
    cfg.frac_inf = c.frac_inf;
    cfg.frac_lwl = c.frac_lwl;
    cfg.ev_wl_min = c.ev_wl_min;
    sw2d_handle* h = nullptr;
    check(sw2d_create(&cfg, &h), "sw2d_create");
    struct Closer {
        sw2d_handle* h;
        ~Closer() { sw2d_destroy(h); }
    } closer{h};
    check(sw2d_set_dem(h, c.dem.data()), "sw2d_set_dem");
    check(sw2d_set_rain_series(h, c.rain.data(), (int)c.rain.size(), c.dtrain), "sw2d_set_rain_series");
    if (c.evaporation_on == 1)
        check(sw2d_set_evaporation_series(h, c.evap.data(), (int)c.evap.size()), "sw2d_set_evaporation_series");
    if (!c.src_cells.empty())
        check(sw2d_set_point_sources(h, (int)c.src_cells.size(), c.src_cells.data(), c.src_q.data(), c.nq, c.dtoq),
              "sw2d_set_point_sources");
    check(sw2d_set_depth(h, c.h0.data()), "sw2d_set_depth");
    int nfaces = 0;
    std::vector<int> fside, fi, fj, fcell;
    if (coupled) {
        check(sw2d_set_coupling_mask(h, c.mask.data(), 1, &nfaces), "sw2d_set_coupling_mask");
        fside.resize(nfaces);
        fi.resize(nfaces);
        fj.resize(nfaces);
        fcell.resize(nfaces);
        if (nfaces > 0)
            check(sw2d_get_coupling_faces(h, fside.data(), fi.data(), fj.data(), fcell.data(), nfaces),
                  "sw2d_get_coupling_faces");
        /* the cards listing the inflow faces (SW2D-EFDC.cu:4919-4930) */
        check(sw2d_write_efdc_cards(join(efdc_dir, "EFDC.INP").c_str(), nfaces, fside.data(), fi.data(), fj.data(),
                                    (int)c.s2v("salt_on"), (int)c.s2v("temp_on"), (int)c.s2v("dye_on")),
              "sw2d_write_efdc_cards");
    }
    /* outlets in the order the reference finds them: by raster id, then by
     * their order in coord_out.dat (SW2D-EFDC.cu:4981-5010) */
    std::vector<std::pair<long long, int>> outlets;
    for (int k = 0; k < (int)c.outlet_cell.size(); k++)
        if (c.outlet_cell[k] >= 0) outlets.push_back({c.outlet_cell[k], k});
    std::sort(outlets.begin(), outlets.end());

    std::vector<double> depth(c.cells()), uu, vv;
    if (c.out_vx == 1 || c.out_vy == 1) {
        uu.resize(c.cells());
        vv.resize(c.cells());
    }
    std::vector<double> qs, times;
    std::vector<double> qrow(nfaces);
    const auto wall0 = std::chrono::steady_clock::now();
    long long done = 0;
    size_t pi = 0;
    auto flush_prints = [&](long long upto) {
        for (; pi < prints.size() && prints[pi].first <= upto; pi++)
            if (!o.quiet) std::printf(" %d\n", prints[pi].second);
        std::fflush(stdout);
    };
    auto advance_to = [&](long long target) {
        /* bounded chunks so that progress lines come out as the run goes */
        while (done < target) {
            const long long n = std::min<long long>(target - done, 2048);
            check(sw2d_step(h, (int)n, c.timmax), "sw2d_step");
            done += n;
            flush_prints(done);
        }
    };
    std::string tempo;
    int tq = -1;
    for (const Event& e : ev) {
        advance_to(e.iteration);
        tq++;
        tempo = e.tempo;
        const bool first = e.iteration == 1; /* the reference's out0 == 0: depths as read */
        if (coupled) {
            /* the first sample reads the initial depths with zero velocities,
             * later ones the velocities of the sample before (SW2D-EFDC.cu:4904-4916) */
            if (nfaces > 0) check(sw2d_couple_sample(h, tq == 0, qrow.data(), nfaces), "sw2d_couple_sample");
            qs.insert(qs.end(), qrow.begin(), qrow.end());
            times.push_back(tq == 0 ? 0.0 : (double)e.mstep * c.dt / c.s2v("efdc_basetime"));
        }
        FILE* f = open_out(join(out_dir, "Results_" + e.tempo + ".vtk"));
        std::fprintf(f, "%s\n", "# vtk DataFile Version 2.0");
        std::fprintf(f, "%s\n", "Brazil");
        std::fprintf(f, "%s\n", "ASCII");
        std::fprintf(f, "%s\n", "DATASET STRUCTURED_POINTS");
        std::fprintf(f, "DIMENSIONS %d %d %d\n", C, R, 1);
        std::fprintf(f, "ASPECT_RATIO %lf %lf %lf\n", g.cellsize, g.cellsize, 1.0000);
        std::fprintf(f, "ORIGIN %lf %lf %lf\n", g.xll, g.yll, 0.000);
        std::fprintf(f, "POINT_DATA %d\n", C * R);
        if (c.out_depth == 1) {
            const std::vector<double>* d = &c.h0;
            if (!first) {
                check(sw2d_get_state(h, depth.data(), nullptr, nullptr), "sw2d_get_state");
                d = &depth;
            }
            if (c.out_outlet == 1) {
                for (size_t k = 0; k < outlets.size(); k++)
                    std::fprintf(wl, (int)(k + 1) == c.n_out ? " %lf\n" : " %lf", (*d)[(size_t)outlets[k].first]);
            }
            std::fprintf(f, "%s\n", "SCALARS depth float 1");
            std::fprintf(f, "%s\n", "LOOKUP_TABLE default");
            write_field(f, *d, R, C, 1.0);
        }
        if (c.out_vx == 1 || c.out_vy == 1) check(sw2d_get_velocity(h, uu.data(), vv.data()), "sw2d_get_velocity");
        if (c.out_vx == 1) {
            std::fprintf(f, "%s\n", "SCALARS x_velocity float 1");
            std::fprintf(f, "%s\n", "LOOKUP_TABLE default");
            write_field(f, vv, R, C, 1.0);
        }
        if (c.out_vy == 1) {
            std::fprintf(f, "%s\n", "SCALARS y_velocity float 1");
            std::fprintf(f, "%s\n", "LOOKUP_TABLE default");
            write_field(f, uu, R, C, -1.0);
        }
        if (c.out_elev == 1) {
            std::fprintf(f, "%s\n", "SCALARS Elevations float 1");
            std::fprintf(f, "%s\n", "LOOKUP_TABLE default");
            write_field(f, c.dem, R, C, 1.0);
        }
        if (std::ferror(f)) input_error("write failed: Results_" + e.tempo + ".vtk");
        std::fclose(f);
    }
    advance_to(iters);
    if (coupled) {
        const int ns = (int)times.size();
        const int nl = (int)c.s2v("nlayers");
        const double base = c.s2v("efdc_basetime");
        check(sw2d_write_qser(join(efdc_dir, "QSER.INP").c_str(), 0, nl, base, nfaces, fside.data(), ns,
                              times.data(), qs.data()),
              "sw2d_write_qser");
        /* the concentration decks of the same inflows (SW2D-EFDC.cu:5084-5097) */
        if ((int)c.s2v("dye_on") == 1) {
            std::vector<double> v(ns, c.s2v("DYE_IN"));
            check(sw2d_write_efdc_concentration(join(efdc_dir, "DSER.INP").c_str(), 'D', 0, nl, base, nfaces,
                                                fside.data(), ns, times.data(), v.data()),
                  "sw2d_write_efdc_concentration");
        }
        if ((int)c.s2v("temp_on") == 1) {
            if ((int)c.temp.size() < ns) input_error("temperatures.dat: fewer values than coupling samples");
            check(sw2d_write_efdc_concentration(join(efdc_dir, "TSER.INP").c_str(), 'T', 0, nl, base, nfaces,
                                                fside.data(), ns, times.data(), c.temp.data()),
                  "sw2d_write_efdc_concentration");
        }
        if ((int)c.s2v("salt_on") == 1) {
            std::vector<double> v(ns, c.s2v("SALT_IN"));
            check(sw2d_write_efdc_concentration(join(efdc_dir, "SSER.INP").c_str(), 'S', 0, nl, base, nfaces,
                                                fside.data(), ns, times.data(), v.data()),
                  "sw2d_write_efdc_concentration");
        }
        if (!o.quiet)
            std::printf(" EFDC hand-off written (%d boundary faces, %d samples); the lake model itself is not run "
                        "by this driver\n",
                        nfaces, ns);
    }
    const double duration = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
    std::cout << "printf: " << duration << '\n';
    std::cout.flush();
    FILE* t = open_out(join(out_dir, "TimeSimu_" + tempo + ".txt"));
    std::fprintf(t, " %lf\n", duration);
    std::fclose(t);
    std::fclose(wl);
}

int usage() {
    std::fprintf(stderr, "usage: sw2d_cli [--root DIR] [--check] [--fp32] [--device N] [--quiet]\n");
    return 1;
}

} // namespace

int main(int argc, char** argv) {
    Options o;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "--root" && i + 1 < argc) o.root = argv[++i];
        else if (a == "--check") o.check = true;
        else if (a == "--fp32") o.fp32 = true;
        else if (a == "--quiet") o.quiet = true;
        else if (a == "--device" && i + 1 < argc) o.device = std::atoi(argv[++i]);
        else return usage();
    }
    const std::string db = join(o.root, "db");
    try {
        /* db/dir.txt: "dir_number: N" then N case directories (SW2D-EFDC.cu:3734-3736) */
        Reader dir(join(db, "dir.txt"), "db/dir.txt");
        dir.keyword("dir_number:");
        const int n = dir.need_int("dir_number");
        for (int k = 0; k < n; k++) {
            Case c;
            if (!dir.token(&c.name)) input_error("db/dir.txt: fewer case names than dir_number");
            c.dir = join(db, c.name);
            if (!o.check && !o.quiet) std::printf(" SW2D GB300\n CASE: %s\n", c.name.c_str());
            read_setup(c);
            read_inputs(c);
            run_case(c, o);
        }
    } catch (const InputError& e) {
        std::printf("%s\n", e.msg.c_str());
        return 1;
    } catch (const LibError& e) {
        std::fflush(stdout);
        std::fprintf(stderr, "sw2d_cli: %s\n", e.msg.c_str());
        return 2;
    } catch (const std::bad_alloc&) {
        std::fflush(stdout);
        std::fprintf(stderr, "sw2d_cli: out of host memory\n");
        return 2;
    }
    return 0;
}
