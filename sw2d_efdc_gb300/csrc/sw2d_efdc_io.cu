/* EFDC hand-off files written from the coupling samples (host code).
 *
 * QSER.INP is the boundary-inflow time-series deck EFDC reads at
 * EFDC_src/INPUT.F:3969-4010; the reference writes it in write_efdc_QSER
 * (SW2D-EFDC.cu:2499-2610) from its per-side *_bc / *_val arrays, and the
 * dye, temperature and salinity decks of the same inflows in write_efdc_DSER,
 * write_efdc_TSER, write_efdc_SSER (:2383-2498, :2141-2254, :2026-2140).  Here
 * the same decks are written from the face list of sw2d_get_coupling_faces
 * and the samples of sw2d_couple_sample, with the reference's layout and
 * number formats so that the files are byte for byte the same.  The cards of
 * EFDC.INP that list those inflows (C22-C26) are rewritten in place as
 * write_efdc_CONFIG rewrites them (SW2D-EFDC.cu:1476-1766). */
#include "sw2d.h"

#include <algorithm>
#include <cstdarg>
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

int io_error(const char* what, const char* path) {
    sw2d::set_error_message((std::string(what) + path).c_str());
    return SW2D_ERR_IO;
}

/* ---- EFDC.INP cards C22-C26 ---------------------------------------------
 * The comment lines of each card are EFDC.INP's own documentation of the
 * card and are kept as the reference writes them, since the file must come
 * out byte for byte the same (SW2D-EFDC.cu:1496-1516, :1548-1570,
 * :1603-1630, :1699-1709, :1745-1756). */
const char* const kDashes = "-------------------------------------------------------------------------------";

const char* const kCardC22[] = {
    "C22 SPECIFY NUM OF SEDIMENT AND TOXICS AND NUM OF CONCENTRATION TIME SERIES",
    "* ",
    "*  NTOX:   NUMBER OF TOXIC CONTAMINANTS (DEFAULT = 1)",
    "*  NSED:   NUMBER OF COHESIVE SEDIMENT SIZE CLASSES (DEFAULT = 1)",
    "*  NSND:   NUMBER OF NON-COHESIVE SEDIMENT SIZE CLASSES (DEFAULT = 1)",
    "*  NCSER1: NUMBER OF SALINITY TIME SERIES",
    "*  NCSER2: NUMBER OF TEMPERATURE TIME SERIES",
    "*  NCSER3: NUMBER OF DYE CONCENTRATION TIME SERIES",
    "*  NCSER4: NUMBER OF SHELLFISH LARVAE CONCENTRATION TIME SERIES",
    "*  NCSER5: NUMBER OF TOXIC CONTAMINANT CONCENTRATION TIME SERIES",
    "*          EACH TIME SERIES MUST HAVE DATA FOR NTOX TOXICICANTS",
    "*  NCSER6: NUMBER OF COHESIVE SEDIMENT CONCENTRATION TIME SERIES",
    "*          EACH TIME SERIES MUST HAVE DATA FOR NSED COHESIVE SEDIMENTS",
    "*  NCSER7: NUMBER OF NON-COHESIVE SEDIMENT CONCENTRATION TIME SERIES",
    "*          EACH TIME SERIES MUST HAVE DATA FOR NSND NON-COHESIVE SEDIMENTS",
    "*  ISSBAL: SET TO 1 FOR SEDIENT MASS BALANCE           ! JOHN & JI, 4/25/97",
    "*",
    "C22 NTOX    NSED    NSND  NCSER1  NCSER2  NCSER3  NCSER4  NCSER5  NCSER6  NCSER7  ISSBAL",
};

const char* const kCardC23[] = {
    "C23 VELOCITY, VOLUMN SOURCE / SINK, FLOW CONTROL, AND WITHDRAWAL / RETURN DATA",
    "*",
    "*  NVBS:   VEL BC(NOT USED)",
    "*  NUBW : VEL BC(NOT USED)",
    "*  NUBE : VEL BC(NOT USED)",
    "*  NVBN : VEL BC(NOT USED)",
    "*  NQSIJ : NUMBER OF CONSTANT AND / OR TIME SERIES SPECIFIED SOURCE / SINK",
    "*          LOCATIONS(RIVER INFLOWS, ETC)             .",
    "*  NQJPIJ : NUMBER OF CONSTANT AND / OR TIME SERIES SPECIFIED SOURCE",
    "*          LOCATIONS TREATED AS JETS / PLUMES          .",
    "*  NQSER : NUMBER OF VOLUME SOURCE / SINK TIME SERIES",
    "*  NQCTL : NUMBER OF PRESSURE CONTROLED WITHDRAWAL / RETURN PAIRS",
    "*  NQCTLT : NUMBER OF PRESSURE CONTROLED WITHDRAWAL / RETURN TABLES",
    "*  NQWR : NUMBER OF CONSTANT OR TIME SERIES SPECIFIED WITHDRAWL / RETURN",
    "*          PAIRS",
    "*  NQWRSR : NUMBER OF TIME SERIES SPECIFYING WITHDRAWL, RETURN AND",
    "*          CONCENTRATION RISE SERIES",
    "*  ISDIQ : SET TO 1 TO WRITE DIAGNOSTIC FILE, DIAQ.OUT",
    "*",
    "C23 NVBS    NUBW    NUBE    NVBN   NQSIJ  NQJPIJ   NQSER   NQCTL  NQCTLT    NQWR  NQWRSR   ISDIQ",
};

const char* const kCardC24[] = {
    "C24 VOLUMETRIC SOURCE / SINK LOCATIONS, MAGNITUDES, AND CONCENTRATION SERIES",
    "*",
    "*  IQS:      I CELL INDEX OF VOLUME SOURCE / SINK",
    "*  JQS : J CELL INDEX OF VOLUME SOURCE / SINK",
    "*  QSSE : CONSTANT INFLOW / OUTFLOW RATE IN M*m*m / s",
    "*  NQSMUL : MULTIPLIER SWITCH FOR CONSTANT AND TIME SERIES VOL S / S",
    "* = 0  MULT BY 1. FOR NORMAL IN / OUTFLOW(L*L*L / T)",
    "* = 1  MULT BY DY FOR LATERAL IN / OUTFLOW(L*L / T) ON U FACE",
    "* = 2  MULT BY DX FOR LATERAL IN / OUTFLOW(L*L / T) ON V FACE",
    "* = 3  MULT BY DX + DY FOR LATERAL IN / OUTFLOW(L*L / T) ON U&V FACES",
    "*  NQSMFF : IF NON ZERO ACCOUNT FOR VOL S / S MOMENTUM FLUX",
    "* = 1  MOMENTUM FLUX ON NEG U FACE",
    "* = 2  MOMENTUM FLUX ON NEG V FACE",
    "* = 3  MOMENTUM FLUX ON POS U FACE",
    "* = 4  MOMENTUM FLUX ON POS V FACE",
    "*  IQSERQ : ID NUMBER OF ASSOCIATED VOLUMN FLOW TIME SERIES",
    "*  ICSER1 : ID NUMBER OF ASSOCIATED SALINITY TIME SERIES",
    "*  ICSER2 : ID NUMBER OF ASSOCIATED TEMPERATURE TIME SERIES",
    "*  ICSER3 : ID NUMBER OF ASSOCIATED DYE CONC TIME SERIES",
    "*  ICSER4 : ID NUMBER OF ASSOCIATED SHELL FISH LARVAE RELEASE TIME SERIES",
    "*  ICSER5 : ID NUMBER OF ASSOCIATED TOXIC CONTAMINANT CONC TIME SERIES",
    "*  ICSER6 : ID NUMBER OF ASSOCIATED COHESIVE SEDIMENT CONC TIME SERIES",
    "*  ICSER7 : ID NUMBER OF ASSOCIATED NON - COHESIVE SED CONC TIME SERIES",
    "*  QSFACTOR : FRACTION OF TIME SERIES FLOW NQSERQ ASSIGNED TO THIS CELL",
    "*",
    "C24  IQS     JQS     QSSE     NQSMUL  NQSMFF  IQSERQ  ICSER1  ICSER2  ICSER3  ICSER4  ICSER5  ICSER6  ICSER7   "
    "QSFACTOR  !ID",
};

const char* const kCardC25[] = {
    "C25 TIME CONSTANT INFLOW CONCENTRATIONS FOR TIME CONSTANT VOLUMETRIC SOURCES",
    "*",
    "*  SAL: SALT CONCENTRATION CORRESPONDING TO INFLOW ABOVE",
    "*  TEM : TEMPERATURE CORRESPONDING TO INFLOW ABOVE",
    "*  DYE : DYE CONCENTRATION CORRESPONDING TO INFLOW ABOVE",
    "*  SFL : SHELL FISH LARVAE CONCENTRATION CORRESPONDING TO INFLOW ABOVE",
    "*  TOX : NTOX TOXIC CONTAMINANT CONCENTRATIONS CORRESPONDING TO",
    "*       INFLOW ABOVE  WRITTEN AS TOXC(N), N = 1, NTOX A SINGLE DEFAULT",
    "*       VALUE IS REQUIRED EVEN IF TOXIC TRANSPORT IS NOT ACTIVE",
    "*",
    "C25    SAL       TEM       DYE       SFL  !ID",
};

const char* const kCardC26[] = {
    "C26 TIME CONSTANT INFLOW CONCENTRATIONS FOR TIME CONSTANT VOLUMETRIC SOURCES",
    "*",
    "*  SED: NSED COHESIVE SEDIMENT CONCENTRATIONS CORRESPONDING TO",
    "*       INFLOW ABOVE  WRITTEN AS SEDC(N), N = 1, NSED.I.E., THE FIRST",
    "*       NSED VALUES ARE COHESIVE A SINGLE DEFAULT VALUE IS REQUIRED",
    "*       EVEN IF COHESIVE SEDIMENT TRANSPORT IS INACTIVE",
    "*  SND : NSND NON - COHESIVE SEDIMENT CONCENTRATIONS CORRESPONDING TO",
    "*       INFLOW ABOVE  WRITTEN AS SND(N), N = 1, NSND.I.E., THE LAST",
    "*       NSND VALUES ARE NON - COHESIVE.A SINGLE DEFAULT VALUE IS",
    "*       REQUIRED EVEN IF NON - COHESIVE SEDIMENT TRANSPORT IS INACTIVE",
    "*",
    "C26   SED1    SND1",
};

const char* const kBcLabel[4] = {"! North_bc", "! South_bc", "! East_bc", "! West_bc"};

bool is_ws(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r'; }

/* One conversion of the scan the reference finds cards with: skip white
 * space, read a token, take the one character after it and, with skip_ws,
 * the white space after that (fscanf "%s%*c" / "%s%*c\n",
 * SW2D-EFDC.cu:1481, :1489).  False when no token is left. */
bool scan_token(const std::string& b, size_t& p, std::string& tok, bool skip_ws) {
    while (p < b.size() && is_ws((unsigned char)b[p])) p++;
    if (p >= b.size()) return false;
    const size_t s = p;
    while (p < b.size() && !is_ws((unsigned char)b[p])) p++;
    tok.assign(b, s, p - s);
    if (p < b.size()) p++;
    if (skip_ws)
        while (p < b.size() && is_ws((unsigned char)b[p])) p++;
    return true;
}

/* Replace card `card` up to the first token `next` with `text`, the file
 * surgery of each card in write_efdc_CONFIG (e.g. SW2D-EFDC.cu:1476-1527):
 *  - `next` is found scanning with "%s%*c\n"; the tail is the tam - pos_next
 *    bytes (tam = size - 4) read from just after that token's scan;
 *  - `card` is found scanning with "%s%*c"; writing starts where the scan
 *    before it stopped;
 *  - the card text, then `next` and a space, then the tail are written over
 *    the old bytes; the file never shrinks, and the bytes from the end of
 *    the writes up to tam become spaces.
 * Tail bytes beyond the end of the file (a `next` token followed by more than
 * one white-space character) are uninitialised memory in the reference and
 * are written as spaces here. */
int replace_card(std::string& b, const char* card, const char* next, const std::string& text) {
    const long long size = (long long)b.size();
    const long long tam = size - 4;
    std::string tok;
    size_t p = 0;
    long long pos_next = 0;
    bool found = false;
    while (scan_token(b, p, tok, true)) {
        if (tok == next) {
            found = true;
            break;
        }
        pos_next = (long long)p;
    }
    if (!found) return bad((std::string("EFDC.INP has no card ") + next).c_str());
    const long long tamcp = tam - pos_next;
    if (tamcp < 0) return bad("EFDC.INP is shorter than its card layout");
    std::string tail((size_t)tamcp, ' ');
    const size_t avail = b.size() - p;
    b.copy(&tail[0], std::min<size_t>(avail, (size_t)tamcp), p);
    size_t q = 0;
    long long pos_card = 0;
    found = false;
    while (scan_token(b, q, tok, false)) {
        if (tok == card) {
            found = true;
            break;
        }
        pos_card = (long long)q;
    }
    if (!found) return bad((std::string("EFDC.INP has no card ") + card).c_str());
    std::string out = b.substr(0, (size_t)pos_card);
    out += text;
    out += next;
    out += ' ';
    out += tail;
    const long long end = (long long)out.size();
    if (end < size) {
        out.append(b, (size_t)end, std::string::npos);
        for (long long k = end; k < tam; k++) out[(size_t)k] = ' ';
    }
    b.swap(out);
    return SW2D_OK;
}

std::string lines(const char* const* l, size_t n) {
    std::string s;
    for (size_t k = 0; k < n; k++) {
        s += l[k];
        s += '\n';
    }
    return s;
}

std::string format(const char* fmt, ...) __attribute__((format(printf, 1, 2)));
std::string format(const char* fmt, ...) {
    va_list ap, aq;
    va_start(ap, fmt);
    va_copy(aq, ap);
    char buf[512];
    const int n = std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    std::string out;
    if (n >= (int)sizeof buf) { /* a longer line: format it again at its length */
        out.resize((size_t)n + 1);
        std::vsnprintf(&out[0], out.size(), fmt, aq);
        out.resize((size_t)n);
    } else if (n > 0) {
        out.assign(buf, (size_t)n);
    }
    va_end(aq);
    return out;
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

extern "C" int sw2d_write_efdc_cards(const char* path, int n_faces, const int* side, const int* efdc_i,
                                     const int* efdc_j, int salt_on, int temp_on, int dye_on) {
    if (!path || (n_faces > 0 && (!side || !efdc_i || !efdc_j))) return bad("null argument");
    if (n_faces < 0) return bad("n_faces < 0");
    for (int k = 0; k < n_faces; k++)
        if (side[k] < 0 || side[k] > 3) return bad("face side outside 0..3 (north, south, east, west)");
    std::string b;
    {
        FILE* f = std::fopen(path, "rb");
        if (!f) return io_error("cannot open ", path);
        char buf[1 << 16];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) b.append(buf, n);
        const bool ok = std::ferror(f) == 0;
        std::fclose(f);
        if (!ok) return io_error("read failed: ", path);
    }
    const int n = n_faces;
    /* C22: salinity, temperature and dye series, one per face where switched on */
    std::string c22 = "\n" + lines(kCardC22, sizeof kCardC22 / sizeof *kCardC22) +
                      format("    %d      %d      %d      %d      %d      %d      %d      %d      %d      %d      %d\n",
                             0, 0, 0, salt_on * n, temp_on * n, dye_on * n, 0, 0, 0, 0, 0) +
                      kDashes + "\n";
    /* C23: NQSIJ sources and NQSER flow series, one of each per face */
    std::string c23 =
        "\n" + lines(kCardC23, sizeof kCardC23 / sizeof *kCardC23) +
        format("    %d      %d      %d      %d      %d      %d      %d      %d      %d      %d     %d      %d\n", 0, 0,
               0, 0, n, 0, n, 0, 0, 0, 0, 0) +
        kDashes + "\n";
    /* C24: a source row per face, numbered across the sides in QSER.INP's order */
    std::string c24 = lines(kCardC24, sizeof kCardC24 / sizeof *kCardC24);
    int nqs = 0;
    for (int s = 0; s < 4; s++)
        for (int k = 0; k < n; k++) {
            if (side[k] != s) continue;
            nqs++;
            c24 += format("     %d      %d      %lf      %d      %d      %d      %d      %d      %d      %d      %d      "
                          "%d      %d      %lf      %s\n",
                          efdc_i[k], efdc_j[k], 0.000, 0, 0, nqs, salt_on * nqs, temp_on * nqs, dye_on * nqs, 0, 0, 0,
                          0, 1.000000, kBcLabel[s]);
        }
    c24 += kDashes;
    c24 += "\n";
    /* C25 and C26: a row of zero constant inflow concentrations and a row of
     * zero sediment concentrations per source */
    std::string c25 = lines(kCardC25, sizeof kCardC25 / sizeof *kCardC25);
    std::string c26 = lines(kCardC26, sizeof kCardC26 / sizeof *kCardC26);
    for (int i = 0; i < nqs; i++) {
        c25 += format("     %lf      %lf      %lf      %lf  %s%d\n", 0.00, 0.00, 0.00, 0.00, "!IQSERQ_", i + 1);
        c26 += format("     %d      %d\n", 0, 0);
    }
    c25 += kDashes;
    c25 += "\n";
    c26 += kDashes;
    c26 += "\n";
    int rc;
    if ((rc = replace_card(b, "C22", "C23", c22)) || (rc = replace_card(b, "C23", "C24", c23)) ||
        (rc = replace_card(b, "C24", "C25", c24)) || (rc = replace_card(b, "C25", "C26", c25)) ||
        (rc = replace_card(b, "C26", "C27", c26)))
        return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return io_error("cannot open ", path);
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    if (std::fclose(f) != 0 || !ok) return io_error("write failed: ", path);
    return SW2D_OK;
}
