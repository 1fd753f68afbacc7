/* Host-side preparation of a case's inputs (no device work):
 *
 *  - sw2d_lake_catchment_smooth: the DEM pre-pass of a coupled run
 *    (lake_catchment_smooth, SW2D-EFDC.cu:2766-2827);
 *  - sw2d_evaporation_series: the evaporation series from temperature and
 *    radiation (gpu_evaporation_calc, SW2D-EFDC.cu:556-586);
 *  - sw2d_manning_classes_of: a per-cell Manning field as a class raster and
 *    the table of its distinct values (the reference has one scalar n).
 *
 * All run once per case over at most rows*cols values.  The smoothing pass
 * stays on the host because its result depends on its sweep order: each
 * cell reads the already-updated cells south and west of it, so a device
 * version would need a wavefront of rows+cols dependent steps for a pass
 * that touches only the cells along the lake edge.  Compiled with
 * -ffp-contract=off: every operation is the single IEEE operation written,
 * as in the CPU build of the reference.
 */
#include "sw2d.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <string>
#include <vector>

namespace sw2d {
void set_error_message(const char* msg); /* sw2d_api.cu */
}

namespace {

/* the literal the reference compares against, whatever the grid's NODATA */
constexpr double kRefNodata = -9999.0;

int bad(const char* msg) {
    sw2d::set_error_message(msg);
    return SW2D_ERR_INVALID;
}

} // namespace

extern "C" int sw2d_lake_catchment_smooth(int rows, int cols, const int* mask, double* dem) {
    if (!mask || !dem) return bad("null argument");
    if (rows < 1 || cols < 1) return bad("rows and cols must be >= 1");
    const ptrdiff_t C = cols;
    /* rows from the last raster row (south) to the first, each west to east;
     * edge rows and columns are left as they are */
    for (int r = rows - 2; r >= 1; r--)
        for (int c = 1; c < cols - 1; c++) {
            const ptrdiff_t k = (ptrdiff_t)r * C + c;
            const int m = mask[k];
            if (m == 1) continue;
            double* z = dem;
            /* across the edge with the row above, then below, then the
             * columns west and east: each test may overwrite the last */
            if (m != mask[k - C] && z[k + C] != kRefNodata) z[k] = (z[k - C] + z[k + C]) / 2.0;
            if (m != mask[k + C] && z[k - C] != kRefNodata) z[k] = (z[k - C] + z[k + C]) / 2.0;
            if (m != mask[k - 1] && z[k + 1] != kRefNodata) z[k] = (z[k - 1] + z[k + 1]) / 2.0;
            if (m != mask[k + 1] && z[k - 1] != kRefNodata) z[k] = (z[k - 1] + z[k + 1]) / 2.0;
        }
    return SW2D_OK;
}

extern "C" int sw2d_evaporation_series(int n, const double* temp, const double* rad, double albedo,
                                       double dtrain, double* mm_out) {
    if (n < 0) return bad("n < 0");
    if (n > 0 && (!temp || !rad || !mm_out)) return bad("null argument");
    for (int i = 0; i < n; i++) {
        const double T = temp[i];
        /* net radiation, W/m2 */
        const double rs = (1 - albedo) * rad[i];
        /* water density, kg/m3: ITS-90 polynomial in T (5-40 deg C) */
        const double pw = 999.85308 + 6.32693 * (0.01) * T - 8.523829 * (0.001) * T * T +
                          6.943248 * (0.00001) * T * T * T - 3.821216 * (0.0000001) * T * T * T * T;
        /* latent heat of vaporisation, J/kg (Henderson-Sellers 1984) */
        const double tk = T + 273.15;
        const double ratio = tk / (tk - 33.91);
        const double lv = (ratio * ratio) * 1.91846 * 1000000;
        /* energy-balance evaporation (Chow et al. 1988, 3.5), mm per dtrain */
        const double e = (rs / (lv * pw)) * dtrain * 1000.0;
        mm_out[i] = e < 0 ? 0 : e;
    }
    return SW2D_OK;
}

extern "C" int sw2d_manning_classes_of(int64_t count, const double* field, int max_classes, uint8_t* classes,
                                       double* table, int* ntable_out) {
    if (count < 0 || max_classes < 1 || max_classes > 256) return bad("count >= 0, 1 <= max_classes <= 256");
    if (count > 0 && (!field || !classes || !table)) return bad("null argument");
    std::vector<double> v(field, field + count);
    for (double x : v)
        if (!(x >= 0) || !std::isfinite(x)) return bad("Manning n must be finite and >= 0");
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    if ((int64_t)v.size() > max_classes) {
        sw2d::set_error_message(("Manning field has " + std::to_string(v.size()) + " distinct values, at most " +
                                 std::to_string(max_classes) + " fit the class table")
                                    .c_str());
        return SW2D_ERR_INVALID;
    }
    for (int64_t k = 0; k < count; k++)
        classes[k] = (uint8_t)(std::lower_bound(v.begin(), v.end(), field[k]) - v.begin());
    std::copy(v.begin(), v.end(), table);
    if (ntable_out) *ntable_out = (int)v.size();
    return SW2D_OK;
}
