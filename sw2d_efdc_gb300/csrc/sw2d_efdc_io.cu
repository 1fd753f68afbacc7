/* EFDC hand-off files written from the coupling samples (host code).
 *
 * QSER.INP is the boundary-inflow time-series deck EFDC reads at
 * EFDC_src/INPUT.F:3969-4010; the reference writes it in write_efdc_QSER
 * (SW2D-EFDC.cu:2499-2610) from its per-side *_bc / *_val arrays, and the
 * dye, temperature and salinity decks of the same inflows in write_efdc_DSER,
 * write_efdc_TSER, write_efdc_SSER (:2383-2498, :2141-2254, :2026-2140).  Here
 * the same decks are written from the face list of sw2d_get_coupling_faces
 * and the samples of sw2d_couple_sample, with the reference's layout and
 * number formats so that the files are byte for byte the same. */
#include "sw2d.h"

#include <cstdio>
#include <string>

namespace sw2d {
void set_error_message(const char* msg); /* sw2d_api.cu */
}

namespace {

/* the deck's comment header, line for line as the reader expects it */
const char* const kQserHeader[] = {
    "C **, qser.inp Time Series FILE",
    "C **",
    "C **  InType MQSER(NS) TCQSER(NS) TAQSER(NS) RMULADJ(NS) ADDADJ(NS) ICHGQS",
    "C **",
    "C **  IF InType.EQ.1 THEN READ DEPTH WEIGHTS AND SINGLE VALUE OF QSER",
    "C **                      ELSE READ A VALUE OF QSER FOR EACH LAYER",
    "C **",
    "C **  InType = 1 Structure",
    "C **  WKQ(K), K = 1, KC",
    "C **  TQSER(M, NS)    QSER(M, 1, NS)          !(MQSER(NS) PAIRS FOR NS = 1, NQSER SERIES)",
    "C **",
    "C **  InType = 0 Structure",
    "C **  TQSER(M, NS)    (QSER(M, K, NS), K = 1, KC) !(MQSER(NS) PAIRS)",
    "C **",
};

const char* const kSideLabel[4] = {" ' *** North_edge_", " ' *** South_edge_", " ' *** East_edge_",
                                   " ' *** West_edge_"};

int bad(const char* msg) {
    sw2d::set_error_message(msg);
    return SW2D_ERR_INVALID;
}

} // namespace

extern "C" int sw2d_write_qser(const char* path, int type, int nlayers, double efdc_basetime, int n_faces,
                               const int* side, int nsamples, const double* times, const double* q) {
    if (!path || (n_faces > 0 && (!side || (nsamples > 0 && (!times || !q)))))
        return bad("null argument");
    if (nlayers < 1 || n_faces < 0 || nsamples < 0) return bad("nlayers >= 1, n_faces >= 0, nsamples >= 0");
    for (int k = 0; k < n_faces; k++)
        if (side[k] < 0 || side[k] > 3) return bad("face side outside 0..3 (north, south, east, west)");
    FILE* f = std::fopen(path, "w");
    if (!f) {
        sw2d::set_error_message((std::string("cannot open ") + path).c_str());
        return SW2D_ERR_IO;
    }
    for (const char* line : kQserHeader) std::fprintf(f, "%s\n", line);
    /* one series per face, north faces first, then south, east and west, each
     * side in the order its faces were found; the series are numbered across
     * the sides; each layer carries 1/nlayers of the face's discharge */
    int series = 0;
    for (int s = 0; s < 4; s++)
        for (int k = 0; k < n_faces; k++) {
            if (side[k] != s) continue;
            series++;
            std::fprintf(f, "      %d %d %lf %d %d %d %d %s%d\n", type, nsamples, efdc_basetime, 0, 1, 0, 0,
                         kSideLabel[s], series);
            for (int t = 0; t < nsamples; t++) {
                std::fprintf(f, "      %lf ", times[t]);
                const double v = q[(size_t)t * n_faces + k] / nlayers;
                for (int l = 0; l < nlayers; l++) std::fprintf(f, l == nlayers - 1 ? "%lf\n" : "%lf ", v);
            }
        }
    const bool ok = std::ferror(f) == 0;
    if (std::fclose(f) != 0 || !ok) {
        sw2d::set_error_message((std::string("write failed: ") + path).c_str());
        return SW2D_ERR_IO;
    }
    return SW2D_OK;
}

extern "C" int sw2d_write_efdc_concentration(const char* path, char kind, int type, int nlayers,
                                             double efdc_basetime, int n_faces, const int* side, int nsamples,
                                             const double* times, const double* value) {
    if (kind != 'D' && kind != 'T' && kind != 'S') return bad("kind must be 'D' (dye), 'T' (temperature) or 'S' (salt)");
    if (!path || (n_faces > 0 && (!side || (nsamples > 0 && (!times || !value))))) return bad("null argument");
    if (nlayers < 1 || n_faces < 0 || nsamples < 0) return bad("nlayers >= 1, n_faces >= 0, nsamples >= 0");
    for (int k = 0; k < n_faces; k++)
        if (side[k] < 0 || side[k] > 3) return bad("face side outside 0..3 (north, south, east, west)");
    FILE* f = std::fopen(path, "w");
    if (!f) {
        sw2d::set_error_message((std::string("cannot open ") + path).c_str());
        return SW2D_ERR_IO;
    }
    const char c = kind;
    std::fprintf(f, "C **, %cSER.INP Time Series FILE\n", c);
    std::fprintf(f, "C **\nC **\n");
    std::fprintf(f, "C **  InType M%cSER(NS) TC%cSER(NS) TA%cSER(NS) RMULADJ(NS) ADDADJ(NS)\n", c, c, c);
    std::fprintf(f, "C **\n");
    std::fprintf(f, "C **  IF InType.EQ.1 THEN READ DEPTH WEIGHTS AND SINGLE VALUE OF %cSER\n", c);
    std::fprintf(f, "C **                      ELSE READ A VALUE OF %cSER FOR EACH LAYER\n", c);
    std::fprintf(f, "C **\nC **  InType = 1 Structure\nC **  WKQ(K), K = 1, KC\n");
    std::fprintf(f, "C **  T%cSER(M, NS)    %cSER(M, 1, NS) !(M%cSER(NS) PAIRS FOR NS = 1, N%cSER SERIES)\n", c, c, c,
                 c);
    std::fprintf(f, "C **\nC **  InType = 0 Structure\n");
    std::fprintf(f, "C **  T%cSER(M, NS)    (%cSER(M, K, NS), K = 1, KC) !(M%cSER(NS) PAIRS)\n", c, c, c);
    std::fprintf(f, "C **\n");
    /* one series per face in the order of QSER.INP; every layer of sample t
     * carries value[t] (the reference passes one concentration for dye and
     * salt, a series for temperature) */
    int series = 0;
    for (int s = 0; s < 4; s++)
        for (int k = 0; k < n_faces; k++) {
            if (side[k] != s) continue;
            series++;
            std::fprintf(f, "      %d %d %lf %d %d %d %s%d\n", type, nsamples, efdc_basetime, 0, 1, 0, kSideLabel[s],
                         series);
            for (int t = 0; t < nsamples; t++) {
                std::fprintf(f, "      %lf ", times[t]);
                for (int l = 0; l < nlayers; l++) std::fprintf(f, l == nlayers - 1 ? "%lf\n" : "%lf ", value[t]);
            }
        }
    const bool ok = std::ferror(f) == 0;
    if (std::fclose(f) != 0 || !ok) {
        sw2d::set_error_message((std::string("write failed: ") + path).c_str());
        return SW2D_ERR_IO;
    }
    return SW2D_OK;
}
