/* FP32 precision form of the SW2D step on sm_103a: one persistent,
 * row-marching kernel per chunk of iterations.
 *
 * A work item is a 224-column strip x `seg` rows of one scenario, taken by a
 * CTA of four warps.  Thread 0 streams the strip's rows (232 columns with a
 * 4-cell halo) of depth, bed offset and x/y discharges into a two-block
 * ring in shared memory with 2-D TMA loads (cp.async.bulk.tensor, one
 * mbarrier per block, four rows per block).  Each warp owns 64 staged
 * columns, two per lane, of which 56 are its output; it marches down the
 * rows keeping the last four rows of every quantity in registers (vertical
 * neighbours) and exchanging horizontal neighbours by warp shuffles.  For
 * each new row L the warp computes
 *   face velocities of row L                  (hm_hn, uu1_vv1: SW2D-EFDC.cu:362-452)
 *   x and y face discharges of row L-1         (flux: :97-353)
 *   provisional depth of row L-2 -> dry flag   (continuity at t: :602-664)
 *   row L-3: outward faces of dry cells closed (treat_error: :695-725, per face),
 *            final depth at t+dt with a Kahan-compensated increment,
 *            written back with its north and west faces.
 * There is no index arithmetic per cell and no barrier per row; halo rows
 * and columns are recomputed instead of exchanged, so an iteration reads
 * every field once from HBM and writes it once.  CTAs take work items of
 * every scenario and iteration of the chunk from a device queue; the CTA
 * that finishes a scenario's last item of an iteration reduces its partials
 * in a fixed order, prepares the scenario's next iteration (CFL length,
 * rain) and releases it to the items waiting on it (k32_persist).
 *
 * Arithmetic is binary32 except the clock, the ledger and the CFL length
 * (binary64).  Gravity uses (h_e - h_w) + (z_e - z_w) with bed offsets from
 * the tile datum, so no large elevations are added to small depths.
 */
#include "sw2d_fp32.h"
#include "sw2d_math.h"

#include <math.h>
#include <stddef.h>

#include <algorithm>

namespace sw2d {

#define NW M_NW
#define BW M_BW
#define RB M_RB
#define NS M_NS
#define NT M_NT

#define NF 5 /* staged fields: h, z, qx, qy, Kahan compensation (three rows behind) */

struct alignas(128) ClsStage {
    unsigned char v[M_CLSR][M_CLSW]; /* rows L-2 .. L+RB-1 of the block's first row L */
};
struct alignas(128) RwStage {
    float v[M_RWR][BW]; /* rows L-3 .. L+RB-2 */
};

/* the class and rain-weight rings come last, so that the variants without
 * them launch with less shared memory (fp32_smem_bytes_variant) */
struct SmemM {
    alignas(128) float stage[NS][NF][RB][BW];
    unsigned long long bar[NS];
    float ntab[T32_MAXCLASS];
    float dband[M_MAXBANDS][3]; /* datums of the bands the item spans, strips west / own / east */
    double red[NW][4];
    float redf[NW][2];
    int nls;                    /* point sources inside the work item's staged window */
    int srow[T32_MAXSRC], scol[T32_MAXSRC];
    float sq1[T32_MAXSRC], sq2[T32_MAXSRC];
    unsigned q;                 /* queue ticket of the item in hand (~0u: leave) */
    unsigned qn;                /* the ticket drawn ahead for the next item */
    int last;                   /* this CTA finished its scenario's iteration */
    ClsStage cls[NS];
    RwStage rw[NS];
};
static_assert(offsetof(SmemM, stage) % 128 == 0, "TMA alignment");
static_assert(offsetof(SmemM, cls) % 128 == 0 && sizeof(ClsStage) % 128 == 0, "TMA alignment");
static_assert(offsetof(SmemM, rw) % 128 == 0 && sizeof(RwStage) % 128 == 0, "TMA alignment");
static_assert((RB * BW * 4) % 128 == 0, "each staged array is whole 128-byte lines");
static_assert((BW * 4) % 16 == 0, "TMA inner extent must be a multiple of 16 bytes");

size_t fp32_smem_bytes() { return sizeof(SmemM) + 128; }

/* dynamic shared memory of variant k (bit 0 class raster, bit 1 rain weight):
 * the struct up to the last ring the variant uses, plus the alignment slack */
size_t fp32_smem_bytes_variant(int k) {
    const size_t used = (k & 2) ? sizeof(SmemM) : (k & 1) ? offsetof(SmemM, rw) : offsetof(SmemM, cls);
    return used + 128;
}

/* ---------------- TMA and mbarrier (inline PTX) -------------------------- */

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y,
                                            unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(tm), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

/* ---------------- device helpers ---------------------------------------- */

/* binary32 arithmetic from the hardware approximations (relative error a
 * few 2^-23; the precision form does not need IEEE rounding) */
__device__ __forceinline__ float rcpa(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrta(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float lg2a(float x) {
    float r;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2a(float x) {
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float fsqrt(float x) { return sqrta(fmaxf(x, 0.f)); }

__device__ __forceinline__ bool is_act(float z) { return z == z; } /* NaN bed offset = inactive */

/* The lane's two columns (2l, 2l+1) travel as one float2 and most arithmetic
 * is done on the pair with the packed FADD2 / FMUL2 / FFMA2 instructions. */
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.f), a); } /* a - b, one rounding */
__device__ __forceinline__ float2 abs2(float2 a) { return make_float2(fabsf(a.x), fabsf(a.y)); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(rcpa(a.x), rcpa(a.y)); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrta(a.x), sqrta(a.y)); }
/* |a| * b and |a| + b per column (the absolute value rides on the scalar
 * instruction's operand modifier) */
__device__ __forceinline__ float2 absmul2(float2 a, float2 b) { return make_float2(fabsf(a.x) * b.x, fabsf(a.y) * b.y); }
__device__ __forceinline__ float2 absadd2(float2 a, float2 b) { return make_float2(fabsf(a.x) + b.x, fabsf(a.y) + b.y); }

/* a condition per column; the rows' activity and dry flags travel between
 * rows as 2-bit ints (bit k = column k) */
struct B2 {
    bool x, y;
};
__device__ __forceinline__ B2 operator&(B2 a, B2 b) { return {a.x && b.x, a.y && b.y}; }
__device__ __forceinline__ B2 operator|(B2 a, B2 b) { return {a.x || b.x, a.y || b.y}; }
__device__ __forceinline__ B2 andnot(B2 a, B2 b) { return {a.x && !b.x, a.y && !b.y}; }
__device__ __forceinline__ B2 bits2(int m) { return {(m & 1) != 0, (m & 2) != 0}; }
__device__ __forceinline__ int mask2(B2 m) { return (m.x ? 1 : 0) | (m.y ? 2 : 0); }
__device__ __forceinline__ bool any2(B2 m) { return m.x || m.y; }
__device__ __forceinline__ float2 sel2(B2 m, float2 a, float2 b) { return make_float2(m.x ? a.x : b.x, m.y ? a.y : b.y); }
__device__ __forceinline__ B2 ge2(float2 a, float t) { return {a.x >= t, a.y >= t}; }
__device__ __forceinline__ B2 gt2(float2 a, float t) { return {a.x > t, a.y > t}; }
__device__ __forceinline__ B2 lt2(float2 a, float t) { return {a.x < t, a.y < t}; }
__device__ __forceinline__ B2 act2(float2 z) { return {is_act(z.x), is_act(z.y)}; }

/* hm^-1.3333330 = 2^(-1.3333330 log2 hm), the friction power (SW2D-EFDC.cu:193) */
__device__ __forceinline__ float2 rpow_manning2(float2 hm) {
    const float2 e = mul2(make_float2(lg2a(hm.x), lg2a(hm.y)), f2(-1.3333330f));
    return make_float2(ex2a(e.x), ex2a(e.y));
}

/* value of the neighbouring column on the left / right */
__device__ __forceinline__ float2 left2(float2 v) { return make_float2(__shfl_up_sync(0xffffffffu, v.y, 1), v.x); }
__device__ __forceinline__ float2 right2(float2 v) { return make_float2(v.y, __shfl_down_sync(0xffffffffu, v.x, 1)); }
__device__ __forceinline__ int leftbits(int v) { /* bit k = column k; returns the left neighbours' bits */
    const int up = __shfl_up_sync(0xffffffffu, v, 1);
    return ((up >> 1) & 1) | ((v & 1) << 1);
}
__device__ __forceinline__ int rightbits(int v) {
    const int dn = __shfl_down_sync(0xffffffffu, v, 1);
    return ((v >> 1) & 1) | ((dn & 1) << 1);
}

/* Upwind donor-cell transport across the edge between two faces of the same
 * orientation (the reference's umr/uml, umu/umd, vnr/vnl, vnu/vnd terms,
 * SW2D-EFDC.cu:171-189, :288-306): with w = half the mean of the two face
 * velocities, w (q1 + q0) + |w| (q0 - q1), q0 on the upstream-indexed face.
 * Each edge is shared by the two faces it separates, so it is computed once. */
__device__ __forceinline__ float2 edge2(float2 w, float2 q0, float2 q1) {
    return fma2(w, add2(q1, q0), absmul2(w, sub2(q0, q1)));
}

/* Weir and dry-bed discharges of one face (SW2D-EFDC.cu:125-157), for the
 * faces where the water surface on one side is below the other side's bed
 * or exactly one side is wet; dz = z_e - z_w is the face's bed step. */
__device__ __forceinline__ float face_special(float hw, float he, float dz, float th, float g) {
    const bool d1a = he + dz < 0.f, d1b = hw - dz < 0.f; /* surface e below bed w / surface w below bed e */
    const float hup = d1a ? hw : he;
    const float fw = (hup > th) ? (d1a ? 0.5440f : -0.544f) * hup * fsqrt(g * hup) : 0.f;
    const float hh3 = fmaxf(he + dz, hw) - fmaxf(dz, 0.f); /* higher surface above the higher bed */
    const float fd =
        ((he > 0.f) || (hw > 0.f)) ? -copysignf(0.350f, (he - th) - (hw - th)) * hh3 * fsqrt(2.f * g * hh3) : 0.f;
    return (d1a || d1b) ? fw : fd;
}

struct Face2 {
    float2 hw, he;         /* the two cells' depths (w: north / west, e: south / east) */
    float2 dz;             /* bed step z_e - z_w */
    float2 q0, u0, vt;     /* old discharge, face velocity, cross velocity at the face */
    float2 conv;           /* along + across convection, already scaled */
    float2 fr;             /* -dt2/2 * g * n_face^2 */
    int act;               /* both cells active, per column */
};

/* One face pair of the reference's flux (SW2D-EFDC.cu:110-202 x, :228-319 y)
 * in binary32.  The momentum update (gravity, convection, semi-implicit
 * Manning friction) is evaluated for both columns; the weir / dry-bed forms
 * only when some lane of the warp needs them. */
__device__ __forceinline__ float2 face_flux2(const Face2& f, float th, float g, float gdt2n) {
    const float2 hm = mul2(add2(f.he, f.hw), f2(0.5f));
    const float2 grav = mul2(mul2(f2(gdt2n), hm), add2(sub2(f.he, f.hw), f.dz));
    const float2 sq = sqrt2(fma2(f.u0, f.u0, mul2(f.vt, f.vt)));
    float2 an = mul2(mul2(f.fr, sq), rpow_manning2(hm)); /* -dt2/2 * friction */
    an = sel2(gt2(hm, th), an, f2(0.f));
    const float2 num = sub2(fma2(an, f.q0, f.q0), add2(f.conv, grav));
    const float2 fm = mul2(num, rcp2(sub2(f2(1.f), an)));
    /* which form applies (SW2D-EFDC.cu:115-165) */
    const B2 wet = gt2(f.hw, th) | gt2(f.he, th);
    const B2 d1a = lt2(add2(f.he, f.dz), 0.f);
    const B2 d1b = lt2(sub2(f.hw, f.dz), 0.f);
    const B2 d2 = lt2(mul2(sub2(f.he, f2(th)), sub2(f.hw, f2(th))), 0.f);
    const B2 open = bits2(f.act) & wet;
    const B2 special = open & (d1a | d1b | d2);
    float2 F = sel2(andnot(open, special), fm, f2(0.f));
    if (__any_sync(0xffffffffu, any2(special))) {
        const float sx = face_special(f.hw.x, f.he.x, f.dz.x, th, g);
        const float sy = face_special(f.hw.y, f.he.y, f.dz.y, th, g);
        F = sel2(special, make_float2(sx, sy), F);
    }
    return F;
}

/* ---------------- the row-marching step ---------------------------------- */

/* CLS: the scenario has a Manning-class raster; RW: a rain-weight field;
 * LAKE: lake cells (depth > ev_wl_min) lose a different fraction of the rain
 * than land cells, or evaporate (the per-cell ledger is then kept too);
 * SRC: point sources. */
/* The slot of a scenario's iteration, read past L1: the CTA that reduced the
 * scenario's previous iteration (on any SM) wrote it during this launch. */
__device__ __forceinline__ Slot32 load_slot(const Clock32* clk) {
    Slot32 s;
    const int4* src = reinterpret_cast<const int4*>(&clk->slot);
    int4* dst = reinterpret_cast<int4*>(&s);
#pragma unroll
    for (int k = 0; k < (int)(sizeof(Slot32) / 16); k++) dst[k] = __ldcg(src + k);
    return s;
}
static_assert(sizeof(Slot32) % 16 == 0 && offsetof(Clock32, slot) == 0, "slot read as int4");

/* One work item: a strip of one scenario over `seg` rows, one iteration.
 * gb counts the staged blocks the CTA has used so far: block b of this item
 * goes to stage (gb + b) % NS and completes that stage's barrier phase
 * (gb + b) / NS, so the barriers, initialised once per CTA, keep their
 * phases from item to item (an mbarrier is never re-initialised while the
 * copy engine may still hold state for it).  Returns false when a staged
 * load did not arrive in time (the status bit is set; the launch's results
 * are void). */
template <bool CLS, bool RW, bool LAKE, bool SRC>
__device__ __forceinline__ bool march_item(SmemM& S, const Scn32& P, const int4 w, Part32* __restrict__ part,
                                           unsigned& gb) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    Clock32* clk = P.clk;
    const Slot32 sl = load_slot(clk);
    if (!sl.active) {
        if (tid == 0) {
            Part32 zp = {};
            part[w.w] = zp;
        }
        return true;
    }
    const int cur = sl.cur, nxt = cur ^ 1;
    const int R = P.R, C = P.C, Pp = P.P;
    const int strip = w.y, seg = w.z;
    const int c0 = strip * M_CW;             /* first output column of the strip */
    const int rs = seg * P.seg, re = min(rs + P.seg, R);
    const int Ls = rs - 3;                   /* first staged row */
    const int nblk = (re - rs + 6 + RB - 1) / RB;

    if ((smem_addr(&S.stage[0][0][0][0]) & 127u) != 0u) {
        if (tid == 0) {
            atomicOr(&clk->status, 4);
            Part32 zp = {};
            part[w.w] = zp;
        }
        return true; /* tile skipped, status bit 2 */
    }
    if (tid < T32_MAXCLASS) S.ntab[tid] = P.ntab[tid];
    if (SRC && warp == 0) {
        /* the point sources inside the staged window (rows rs-3 .. re+2,
         * the strip's staged columns), in source order */
        int n = 0;
        for (int k0 = 0; k0 < P.nsrc; k0 += 32) {
            const int k = k0 + lane;
            int r = 0, c = 0;
            bool in = false;
            if (k < P.nsrc) {
                const int cell = P.src_cell[k];
                r = cell / C;
                c = cell - r * C;
                in = r >= rs - 3 && r < re + 3 && c >= c0 - M_H && c < c0 - M_H + BW;
            }
            const unsigned b = __ballot_sync(0xffffffffu, in);
            if (in) {
                const int at = n + __popc(b & ((1u << lane) - 1u));
                S.srow[at] = r;
                S.scol[at] = c;
                S.sq1[at] = __ldcg(&clk->ql1[k]);
                S.sq2[at] = __ldcg(&clk->ql2[k]);
            }
            n += __popc(b);
        }
        if (lane == 0) S.nls = n;
    }
    /* datums of the bands the staged rows span, for the strips west, own
     * and east (0 outside the raster) */
    if (tid < 3 * M_MAXBANDS) {
        const int b0 = max(Ls, 0) / M_DR;
        const int j = tid / 3, cr = tid - 3 * j, nx = strip + cr - 1;
        S.dband[j][cr] = (nx >= 0 && nx < P.tiles_x && b0 + j < P.bands) ? P.datum[(b0 + j) * P.tiles_x + nx] : 0.f;
    }
    __syncthreads();
    constexpr bool has_cls = CLS, has_rw = RW;
    const unsigned blk_bytes = (unsigned)NF * RB * BW * 4u + (has_cls ? (unsigned)(M_CLSR * M_CLSW) : 0u) +
                               (has_rw ? (unsigned)(M_RWR * BW * 4) : 0u);
    /* block b holds rows Ls + b*RB .. +RB-1 of h, z, qx, qy, the Kahan
     * compensation of the rows three above (the rows finished during b) and,
     * when present, the class rows from two above and the rain weights from
     * three above */
    auto issue = [&](int b, int st) {
        mbar_arrive_expect_tx(&S.bar[st], blk_bytes);
        const int y = Ls + b * RB + M_H; /* padded row of the block's first row */
        tma_load_2d(&S.stage[st][0][0][0], &P.tm_h[cur], c0, y, &S.bar[st]);
        tma_load_2d(&S.stage[st][1][0][0], &P.tm_z, c0, y, &S.bar[st]);
        tma_load_2d(&S.stage[st][2][0][0], &P.tm_qx[cur], c0, y, &S.bar[st]);
        tma_load_2d(&S.stage[st][3][0][0], &P.tm_qy[cur], c0, y, &S.bar[st]);
        tma_load_2d(&S.stage[st][4][0][0], &P.tm_kc, c0, y - 3, &S.bar[st]);
        if (has_cls) tma_load_2d(&S.cls[st].v[0][0], &P.tm_cls, c0, y - 2, &S.bar[st]);
        if (has_rw) tma_load_2d(&S.rw[st].v[0][0], &P.tm_rw, c0, y - 3, &S.bar[st]);
    };
    if (tid == 0 && !P.stall_staging) {
        /* the staging buffers were last read by the generic proxy */
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        for (int b = 0; b < NS && b < nblk; b++) issue(b, (int)((gb + b) % NS));
    }

    /* lane geometry: staged columns sc, sc+1; global columns cg, cg+1 */
    const int sc = warp * M_SW + 2 * lane;
    const int cg = c0 - M_H + sc;
    const bool own0 = (lane >= 2 && lane < 30) && cg < C;
    const bool own1 = (lane >= 2 && lane < 30) && cg + 1 < C;
    const int ownm = (own0 ? 1 : 0) | (own1 ? 2 : 0);
    /* the lane's two columns lie in one datum column (strip west, own, east:
     * strips start on even columns); the lanes whose first column starts a
     * datum column see a datum step across their west y face */
    const int creg = sc < M_H ? 0 : (sc >= M_H + M_CW ? 2 : 1);
    const bool yedge = (sc == M_H || sc == M_H + M_CW) && cg > 0;
    const float th = P.th, gg = P.g;
    const float dt2 = sl.dt2, dt2dx = sl.dt2dx, dt2dy = sl.dt2dy;
    const float gdx = gg * dt2dx, gdy = gg * dt2dy;
    const float2 rdxy = make_float2(P.rdx, P.rdy);
    const float n_uni = S.ntab[0];
    const float fr_scale = -0.5f * dt2 * gg;          /* an = fr_scale * n^2 * sq * hm^-4/3 */
    const float fr_uni = fr_scale * n_uni * n_uni;
    /* source terms: rain rate * runoff fraction, evaporation on lake cells */
    const float ewl = P.ev_wl_min;
    const float rl1 = sl.rr1 * P.pct_lake, rd1 = sl.rr1 * P.pct_land;
    const float rl2 = sl.rr2 * P.pct_lake, rd2 = sl.rr2 * P.pct_land;
    const float ev1 = sl.ev1, ev2 = sl.ev2;
    constexpr bool lakefx = LAKE;
    /* the cross convection of x faces vanishes on column 0 (SW2D-EFDC.cu:164) */
    const float2 colm = make_float2(cg == 0 ? 0.f : 1.f, cg + 1 == 0 ? 0.f : 1.f);

    /* register windows, slot = (row - Ls) & 3 */
    float2 H[4], DZX[4], QX[4], QY[4], U[4], UU[4], V[4], VV[4], VR[4];
    float2 HL[4], DZY[4], EX[4], GY[4], FX[4], FY[4], FYR[4];
    int ACT[4], ACTL[4], DRY[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        H[k] = DZX[k] = QX[k] = QY[k] = U[k] = UU[k] = V[k] = VV[k] = VR[k] = f2(0.f);
        HL[k] = DZY[k] = EX[k] = GY[k] = FX[k] = FY[k] = FYR[k] = f2(0.f);
        ACT[k] = ACTL[k] = DRY[k] = 0;
    }
    float2 Zp = f2(0.f); /* bed offsets of the row above */
    /* datum band of the row in hand, counted from the band of the first staged
     * row; it grows by one at each band edge (rows past the last band are
     * the halo, whose bed is NaN whatever its datum) */
    int bj = 0;
    float clamp = 0.f, qout = 0.f, rainacc = 0.f, evc = 0.f;
    float sxm = 0.f, sym = 0.f;
    const int nls = SRC ? S.nls : 0;
    /* point-source rates of the lane's two cells in row `row` (distinct cells) */
    auto point_src = [&](int row, const float* q) {
        float2 v = f2(0.f);
        for (int k = 0; k < nls; k++)
            if (S.srow[k] == row) {
                if (S.scol[k] == cg) v.x += q[k];
                if (S.scol[k] == cg + 1) v.y += q[k];
            }
        return v;
    };

    for (int b = 0; b < nblk; b++) {
        const int st = (int)((gb + b) % NS);
        /* bounded wait for the block (about 2^31 cycles); the CTA agrees on
         * the outcome so that no warp is left waiting at a barrier */
        {
            const unsigned par = ((gb + b) / NS) & 1u;
            long long t0 = clock64();
            bool ok = true;
            while (!mbar_try_wait(&S.bar[st], par)) {
                if (clock64() - t0 > (1ll << 31)) {
                    ok = false;
                    break;
                }
            }
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicOr(&clk->status, 2);
                    /* Blocks b .. b+NS-1 were issued (none under the staging
                     * stall of the failure test) and their loads may still
                     * be in flight into this CTA's shared memory: wait for
                     * them, again bounded, before the CTA exits and its
                     * shared memory is handed to another CTA.  The launch's
                     * results are void either way (status bit 1). */
                    const int issued = P.stall_staging ? 0 : min(nblk, b + NS);
                    for (int bb = b; bb < issued; bb++) {
                        const long long t1 = clock64();
                        while (!mbar_try_wait(&S.bar[(gb + bb) % NS], ((gb + bb) / NS) & 1u) &&
                               clock64() - t1 <= (1ll << 31)) {
                        }
                    }
                }
                return false;
            }
        }
        const float* sh = &S.stage[st][0][0][0];
        const float* sz = &S.stage[st][1][0][0];
        const float* sqx = &S.stage[st][2][0][0];
        const float* sqy = &S.stage[st][3][0][0];
        const float* skc = &S.stage[st][4][0][0];
        const unsigned char* scl = &S.cls[st].v[0][0];
        const float* srw = &S.rw[st].v[0][0];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            const int L = Ls + b * RB + j;
            const int s0 = j & 3, s1 = (j + 3) & 3, s2 = (j + 2) & 3, s3 = (j + 1) & 3; /* L, L-1, L-2, L-3 */
            /* ---- row L from the staged block ---- */
            const float2 h0 = *reinterpret_cast<const float2*>(sh + j * BW + sc);
            const float2 z0 = *reinterpret_cast<const float2*>(sz + j * BW + sc); /* offsets from the band datum */
            const float2 qx0 = *reinterpret_cast<const float2*>(sqx + j * BW + sc);
            const float2 qy0 = *reinterpret_cast<const float2*>(sqy + j * BW + sc);
            H[s0] = h0;
            QX[s0] = qx0;
            QY[s0] = qy0;
            ACT[s0] = mask2(act2(z0));
            const float2 hl = left2(h0);
            HL[s0] = hl;
            ACTL[s0] = leftbits(ACT[s0]);
            /* bed steps of the x face north of row L and the y faces west of
             * its cells, plus the datum step where the face crosses a datum
             * tile's edge (a band edge above row L, a strip edge west) */
            float2 dzx = sub2(z0, Zp);
            if ((L & (M_DR - 1)) == 0 && L > 0) { /* a band edge above row L */
                bj++;
                const float c = S.dband[bj][creg] - S.dband[bj - 1][creg];
                dzx = add2(dzx, f2(c));
            }
            DZX[s0] = dzx;
            Zp = z0;
            float2 dzy = sub2(z0, left2(z0));
            if (yedge) dzy.x += S.dband[bj][creg] - S.dband[bj][creg - 1];
            DZY[s0] = dzy;
            /* ---- face velocities of row L (uu1 at the x face north, vv1 at the y face west) ---- */
            const float2 hm = (L == R) ? H[s1] : mul2(add2(h0, H[s1]), f2(0.5f));
            const float2 hn = mul2(add2(h0, hl), f2(0.5f));
            const B2 okm = ge2(hm, th), okn = ge2(hn, th);
            const float2 u = sel2(okm, mul2(qx0, rcp2(hm)), f2(0.f));
            const float2 v = sel2(okn, mul2(qy0, rcp2(hn)), f2(0.f));
            U[s0] = u;
            V[s0] = v;
            const float2 ul = left2(u), vr = right2(v);
            UU[s0] = add2(u, ul);
            VV[s0] = add2(v, vr);
            VR[s0] = vr;
            /* CFL face speeds (|velocity| + sqrt(g h)) of the owned faces */
            if (L >= rs && L < re) {
                const float2 cx = sel2(okm & bits2(ownm & ACT[s0] & ACT[s1]), absadd2(u, sqrt2(mul2(f2(gg), hm))), f2(0.f));
                const float2 cy = sel2(okn & bits2(ownm & ACT[s0] & ACTL[s0]), absadd2(v, sqrt2(mul2(f2(gg), hn))), f2(0.f));
                sxm = fmaxf(sxm, fmaxf(cx.x, cx.y));
                sym = fmaxf(sym, fmaxf(cy.x, cy.y));
            }
            /* ---- edge terms of the convection ---- */
            EX[s1] = edge2(mul2(add2(u, U[s1]), f2(0.25f)), QX[s1], qx0);
            GY[s1] = edge2(mul2(UU[s0], f2(0.25f)), QY[s1], qy0);
            const float2 EY = edge2(mul2(VV[s1], f2(0.25f)), QY[s1], right2(QY[s1]));
            const float2 GX = edge2(mul2(add2(VR[s1], VR[s2]), f2(0.25f)), QX[s1], right2(QX[s1]));
            /* ---- face discharges of row L-1 ---- */
            const int rf = L - 1;
            {
                Face2 f;
                f.hw = H[s2];
                f.he = H[s1];
                f.dz = DZX[s1];
                f.act = ACT[s2] & ACT[s1];
                f.q0 = QX[s1];
                f.u0 = U[s1];
                f.vt = mul2(add2(VV[s1], VV[s2]), f2(0.25f));
                f.conv = fma2(sub2(EX[s1], EX[s2]), f2(dt2dx), mul2(mul2(sub2(GX, left2(GX)), f2(dt2dy)), colm));
                if (has_cls) { /* face n = mean of the two cells' n; class rows L-2, L-1 at j, j+1 */
                    const unsigned char* c1 = scl + (j + 1) * M_CLSW + sc;
                    const unsigned char* c2 = scl + j * M_CLSW + sc;
                    const float2 nf = mul2(add2(make_float2(S.ntab[c1[0] & 63], S.ntab[c1[1] & 63]),
                                                make_float2(S.ntab[c2[0] & 63], S.ntab[c2[1] & 63])),
                                           f2(0.5f));
                    f.fr = mul2(mul2(nf, nf), f2(fr_scale));
                } else {
                    f.fr = f2(fr_uni);
                }
                float2 F = face_flux2(f, th, gg, gdx);
                if (rf == R) { /* south edge: free overfall when open (SW2D-EFDC.cu:131 law) */
                    const float2 hw = f.hw;
                    const B2 m = bits2(P.outflow_south ? ACT[s2] : 0) & gt2(hw, th);
                    F = sel2(m, mul2(mul2(f2(0.5440f), hw), sqrt2(mul2(f2(gg), hw))), f2(0.f));
                }
                FX[s1] = F;
            }
            {
                Face2 f;
                f.hw = HL[s1];
                f.he = H[s1];
                f.dz = DZY[s1];
                f.act = ACTL[s1] & ACT[s1];
                f.q0 = QY[s1];
                f.u0 = V[s1];
                f.vt = mul2(add2(UU[s1], UU[s0]), f2(0.25f));
                const float2 along = mul2(sub2(EY, left2(EY)), f2(dt2dy));
                f.conv = (rf == 0) ? along : fma2(sub2(GY[s1], GY[s2]), f2(dt2dx), along);
                if (has_cls) { /* row L-1, columns c-1, c, c+1 (sc >= 0 and row j+1 >= 1 keep c-1 inside) */
                    const unsigned char* c1 = scl + (j + 1) * M_CLSW + sc;
                    const float nl = S.ntab[c1[-1] & 63], n0 = S.ntab[c1[0] & 63], n1 = S.ntab[c1[1] & 63];
                    const float2 nf = mul2(add2(make_float2(n0, n1), make_float2(nl, n0)), f2(0.5f));
                    f.fr = mul2(mul2(nf, nf), f2(fr_scale));
                } else {
                    f.fr = f2(fr_uni);
                }
                FY[s1] = face_flux2(f, th, gg, gdy);
            }
            /* ---- provisional depth of row L-2 -> dry flags ---- */
            FYR[s2] = right2(FY[s2]);
            {
                const float2 ho = H[s2];
                float2 src = f2(rd1);
                B2 lake = {false, false};
                if (lakefx) {
                    lake = gt2(ho, ewl);
                    src = sel2(lake, f2(rl1), src);
                }
                if (has_rw) src = mul2(src, *reinterpret_cast<const float2*>(srw + (j + 1) * BW + sc));
                if (lakefx) src = sub2(src, sel2(lake, f2(ev1), f2(0.f)));
                if (SRC && nls) src = add2(src, point_src(L - 2, S.sq1));
                const float2 div = fma2(sub2(FX[s1], FX[s2]), f2(rdxy.x), mul2(sub2(FYR[s2], FY[s2]), f2(rdxy.y)));
                const float2 hs = fma2(sub2(div, src), f2(-dt2), ho);
                DRY[s2] = ACT[s2] & mask2(lt2(hs, th));
            }
            /* ---- final depth of row L-3 ---- */
            const int r = L - 3;
            /* continuity at t+dt, Kahan-compensated, and write-back of the
             * cell with its north and west faces */
            auto finish = [&](float2 fN, float2 fS, float2 fW, float2 fE) {
                const float2 ho = H[s3];
                const B2 act = bits2(ACT[s3]);
                B2 lake = {false, false};
                float2 src = f2(rd2);
                if (LAKE) {
                    lake = gt2(ho, ewl);
                    src = sel2(lake, f2(rl2), src);
                }
                const float2 wgt = RW ? *reinterpret_cast<const float2*>(srw + j * BW + sc) : f2(1.f);
                if (RW) src = mul2(src, wgt);
                if (LAKE) src = sub2(src, sel2(lake, f2(ev2), f2(0.f)));
                if (SRC && nls) src = add2(src, point_src(r, S.sq2));
                const float2 div = fma2(sub2(fS, fN), f2(rdxy.x), mul2(sub2(fE, fW), f2(rdxy.y)));
                const float2 dh = mul2(sub2(div, src), f2(-dt2));
                /* Kahan: the increment is small against the depth */
                const float2 kc0 = *reinterpret_cast<const float2*>(skc + j * BW + sc);
                const float2 y = sub2(dh, kc0);
                const float2 t = add2(ho, y);
                float2 kc = sub2(sub2(t, ho), y);
                const B2 pos = ge2(t, 0.f);
                const B2 oa = bits2(ownm) & act;
                {
                    const float2 ng = sel2(andnot(oa, pos), t, f2(0.f));
                    clamp -= ng.x + ng.y;
                }
                if (LAKE) {
                    float2 pw = sel2(lake, f2(P.pct_lake), f2(P.pct_land));
                    if (RW) pw = mul2(pw, wgt);
                    pw = sel2(oa, pw, f2(0.f));
                    rainacc += pw.x + pw.y;
                    const float2 ec = sel2(oa & lake, f2(1.f), f2(0.f));
                    evc += ec.x + ec.y;
                }
                if (r == R - 1) {
                    const float2 qo = sel2(oa, fS, f2(0.f));
                    qout += qo.x + qo.y;
                }
                kc = sel2(act & pos, kc, f2(0.f));
                const float2 hout = sel2(act, make_float2(fmaxf(t.x, 0.f), fmaxf(t.y, 0.f)), f2(0.f));
                const size_t g = (size_t)(r + M_H) * Pp + (cg + M_H);
                if (own1) {
                    *reinterpret_cast<float2*>(P.h[nxt] + g) = hout;
                    *reinterpret_cast<float2*>(P.kc + g) = kc;
                    *reinterpret_cast<float2*>(P.qx[nxt] + g) = fN;
                    *reinterpret_cast<float2*>(P.qy[nxt] + g) = fW;
                    if (r == R - 1) *reinterpret_cast<float2*>(P.qx[nxt] + g + Pp) = fS;
                } else if (own0) {
                    P.h[nxt][g] = hout.x;
                    P.kc[g] = kc.x;
                    P.qx[nxt][g] = fN.x;
                    P.qy[nxt][g] = fW.x;
                    if (r == R - 1) P.qx[nxt][g + Pp] = fS.x;
                }
            };
            if (r >= rs && r < re) {
                const int dc = DRY[s3], dN = DRY[s0], dS = DRY[s2];
                float2 fN = FX[s3], fS = FX[s2], fW = FY[s3], fE = FYR[s3];
                if (__any_sync(0xffffffffu, (dc | dN | dS) != 0)) {
                    /* treat_error (SW2D-EFDC.cu:695-725): no outflow from a
                     * dry cell; a warp-uniform branch taken only near dry
                     * cells, the finish below shared by both paths (one
                     * copy of it per row keeps the unrolled loop small) */
                    const int dW = leftbits(dc), dE = rightbits(dc);
                    const B2 bc = bits2(dc), bN = bits2(dN), bS = bits2(dS), bW = bits2(dW), bE = bits2(dE);
                    const B2 zN = (gt2(fN, 0.f) & bN) | (lt2(fN, 0.f) & bc);
                    const B2 zS = (gt2(fS, 0.f) & bc) | (lt2(fS, 0.f) & bS);
                    const B2 zW = (gt2(fW, 0.f) & bW) | (lt2(fW, 0.f) & bc);
                    const B2 zE = (gt2(fE, 0.f) & bc) | (lt2(fE, 0.f) & bE);
                    fN = sel2(zN, f2(0.f), fN);
                    fS = sel2(zS, f2(0.f), fS);
                    fW = sel2(zW, f2(0.f), fW);
                    fE = sel2(zE, f2(0.f), fE);
                }
                finish(fN, fS, fW, fE);
            }
        }
        __syncthreads(); /* every warp is done with block b */
        if (tid == 0 && b + NS < nblk) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(b + NS, st);
        }
    }
    gb += (unsigned)nblk;

    /* block reductions: warp sums in binary32, across warps in binary64 */
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sxm = fmaxf(sxm, __shfl_xor_sync(0xffffffffu, sxm, o));
        sym = fmaxf(sym, __shfl_xor_sync(0xffffffffu, sym, o));
        clamp += __shfl_xor_sync(0xffffffffu, clamp, o);
        qout += __shfl_xor_sync(0xffffffffu, qout, o);
        rainacc += __shfl_xor_sync(0xffffffffu, rainacc, o);
        evc += __shfl_xor_sync(0xffffffffu, evc, o);
    }
    if (lane == 0) {
        S.red[warp][0] = clamp;
        S.red[warp][1] = qout;
        S.red[warp][2] = rainacc;
        S.red[warp][3] = evc;
        S.redf[warp][0] = sxm;
        S.redf[warp][1] = sym;
    }
    __syncthreads();
    if (tid == 0) {
        Part32 pr = {};
        float mx = 0.f, my = 0.f;
        for (int k = 0; k < NW; k++) {
            pr.clamp += S.red[k][0];
            pr.qout += S.red[k][1];
            pr.rain += S.red[k][2];
            pr.evap += S.red[k][3];
            mx = fmaxf(mx, S.redf[k][0]);
            my = fmaxf(my, S.redf[k][1]);
        }
        pr.sx = mx * rdxy.x; /* rdx > 0: the maximum commutes with the scaling */
        pr.sy = my * rdxy.y;
        part[w.w] = pr; /* the partials stay in scenario order whatever the launch order */
    }
    return true;
}

/* ---------------- per-scenario finalize ---------------------------------- */

__device__ double series_at32(const double* v, int n, double dts, double time, int mode) {
    int it;
    if (mode == 0) {
        if (time <= 1.00) return v[0] * time;
        it = sw2d_series_index(time, dts, n);
        return v[it] + (v[it + 1] - v[it]) / (dts * (time - dts * (it)));
    } else if (mode == 1) {
        it = sw2d_series_index(time, dts, n);
        return v[it] + (v[it + 1] - v[it]) * ((time - dts * (it)) / dts);
    }
    it = sw2d_series_index(time, dts, n);
    return v[it];
}

/* point-source rate (m/s) of source i at time t: the reference's stream_flow
 * interpolation (SW2D-EFDC.cu:531-538) in REFERENCE mode, else LINEAR / STEP */
__device__ float source_at32(const Scn32& P, int i, double time) {
    const double* Q = P.srcq;
    const int ns = P.nsrc;
    double q;
    if (P.series_mode == 0 && time <= 1.00) {
        q = Q[i] * time;
    } else {
        const int it = sw2d_series_index(time, P.dtoq, P.nq);
        const double a = Q[(size_t)it * ns + i], b = Q[(size_t)(it + 1) * ns + i];
        if (P.series_mode == 0)
            q = a + (b - a) / (P.dtoq * (time - P.dtoq * (it)));
        else if (P.series_mode == 1)
            q = a + (b - a) * ((time - P.dtoq * (it)) / P.dtoq);
        else
            q = a;
    }
    return (float)(q / (P.dxd * P.dyd));
}

/* Length and forcing of the iteration starting at time t.  The clock is
 * accessed as volatile: inside a persistent launch the CTA that reduces a
 * scenario's iteration may sit on another SM than the previous one's. */
__device__ void prepare_slot32(const Scn32& P, volatile Clock32* clk, double t, double t_end, double s_max) {
    double dt2, tm;
    int active;
    if (P.dt_mode == 0) {
        /* the reference's time grid: the clock advances by dt twice, as the
         * FP64 path's; only the state update uses dt2 rounded to binary32 */
        const double dt = P.dt_fixed;
        active = (t + dt <= t_end);
        dt2 = 2.0 * dt;
        tm = t + dt;
    } else {
        active = (t < t_end);
        dt2 = s_max > 0 ? fmin(P.dt_max, P.cfl / s_max) : P.dt_max;
        dt2 = (double)(float)dt2;
        if (t + dt2 > t_end) dt2 = t_end - t;
        tm = t + 0.5 * dt2;
    }
    volatile Slot32& s = clk->slot;
    s.active = active;
    s.dt2 = (float)dt2;
    s.dt2dx = (float)(dt2 / P.dxd);
    s.dt2dy = (float)(dt2 / P.dyd);
    s.rr1 = (float)(series_at32(P.rain, P.nrain, P.dtrain, t, P.series_mode) / (P.dtrain * 1000.0));
    s.rr2 = (float)(series_at32(P.rain, P.nrain, P.dtrain, tm, P.series_mode) / (P.dtrain * 1000.0));
    if (P.evap) {
        s.ev1 = (float)(series_at32(P.evap, P.nevap, P.dtrain, t, P.series_mode) / (P.dtrain * 1000.0));
        s.ev2 = (float)(series_at32(P.evap, P.nevap, P.dtrain, tm, P.series_mode) / (P.dtrain * 1000.0));
    } else {
        s.ev1 = s.ev2 = 0.f;
    }
    for (int k = 0; k < P.nsrc; k++) {
        clk->ql1[k] = source_at32(P, k, t);
        clk->ql2[k] = source_at32(P, k, tm);
    }
    clk->dt2 = dt2;
    if (!active) clk->done = 1;
}

/* One scenario's end of iteration, run by the whole CTA: fixed-order sum of
 * its work items' partials (each thread a fixed stride of them, then the
 * warps and the CTA in a fixed order; read past L1: other CTAs wrote them
 * during this launch), then, by thread 0, the ledger, clock, outlet record
 * and the next slot. */
__device__ __noinline__ void finalize_scn(const Scn32& P, const Part32* __restrict__ part, double (*red)[4],
                                          float (*redf)[2]) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    volatile Clock32* clk = P.clk;
    double clamp = 0, qout = 0, rain = 0, evc = 0;
    float sx = 0.f, sy = 0.f;
    for (int k = tid; k < P.nwork; k += NT) {
        const Part32* q = part + P.first_work + k;
        clamp += __ldcg(&q->clamp);
        qout += __ldcg(&q->qout);
        rain += __ldcg(&q->rain);
        evc += __ldcg(&q->evap);
        sx = fmaxf(sx, __ldcg(&q->sx));
        sy = fmaxf(sy, __ldcg(&q->sy));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        clamp += __shfl_down_sync(0xffffffffu, clamp, o);
        qout += __shfl_down_sync(0xffffffffu, qout, o);
        rain += __shfl_down_sync(0xffffffffu, rain, o);
        evc += __shfl_down_sync(0xffffffffu, evc, o);
        sx = fmaxf(sx, __shfl_down_sync(0xffffffffu, sx, o));
        sy = fmaxf(sy, __shfl_down_sync(0xffffffffu, sy, o));
    }
    if (lane == 0) {
        red[warp][0] = clamp;
        red[warp][1] = qout;
        red[warp][2] = rain;
        red[warp][3] = evc;
        redf[warp][0] = sx;
        redf[warp][1] = sy;
    }
    __syncthreads();
    if (tid != 0 || !clk->slot.active) return;
    for (int k = 1; k < NW; k++) {
        clamp += red[k][0];
        qout += red[k][1];
        rain += red[k][2];
        evc += red[k][3];
        sx = fmaxf(sx, redf[k][0]);
        sy = fmaxf(sy, redf[k][1]);
    }
    const float rr2 = clk->slot.rr2, ev2 = clk->slot.ev2;
    const int cur = clk->slot.cur;
    const double dt2 = clk->dt2;
    const double area = P.area;
    const double rain_sum = P.ledger_cells ? rain : P.rain_static;
    clk->rain_in = clk->rain_in + dt2 * (double)rr2 * rain_sum * area;
    clk->evap_out = clk->evap_out + dt2 * (double)ev2 * evc * area;
    double qsrc = 0.0;
    for (int k = 0; k < P.nsrc; k++) qsrc += (double)clk->ql2[k];
    clk->source_in = clk->source_in + dt2 * qsrc * area;
    clk->clamp_gain = clk->clamp_gain + clamp * area;
    const double q_out = qout * P.dyd;
    clk->q_out = q_out;
    clk->outflow = clk->outflow + dt2 * q_out;
    /* the CFL speed of the state this iteration started from */
    const double s_max = (double)sx + (double)sy;
    clk->s_max = s_max;
    if (!isfinite(s_max) || !isfinite(qout)) clk->status = clk->status | 1;
    const double t = (P.dt_mode == 0) ? (clk->t + P.dt_fixed) + P.dt_fixed : clk->t + dt2;
    clk->t = t;
    clk->iters = clk->iters + 1;
    clk->slot.cur = cur ^ 1;
    if (P.outlet) {
        const long long k = clk->outlet_n % P.outlet_cap;
        P.outlet[2 * k] = t;
        P.outlet[2 * k + 1] = q_out;
        clk->outlet_n = clk->outlet_n + 1;
    }
    prepare_slot32(P, clk, t, clk->t_end, s_max);
}

/* ---------------- the persistent launch ---------------------------------- */

__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

/* The queue side of the persistent loop, run by thread 0: the bounded wait
 * of ticket q (drawn ahead, while the CTA worked on its previous item) for
 * its scenario's previous iteration.  Returns the ticket, or ~0u when the
 * CTA is to leave (the queue is empty, or a wait ran out: then the
 * scenario's timeout bit and the abort flag are set).  A waiting ticket only
 * ever waits for smaller tickets, so holding one ticket ahead cannot close a
 * cycle of waits. */
__device__ __noinline__ unsigned wait_ticket(unsigned q, const Scn32* __restrict__ scns,
                                             const int4* __restrict__ work, int nwork, int niter, Ctl32* ctl) {
    const int* done = reinterpret_cast<const int*>(ctl + 1);
    volatile unsigned* abort_flag = &ctl->abort;
    if (q >= (unsigned)nwork * (unsigned)niter || *abort_flag) return ~0u;
    const int it = (int)(q / (unsigned)nwork);
    const int sc = work[q % (unsigned)nwork].x;
    const long long t0 = clock64();
    while (ld_acquire_gpu(&done[sc]) < it) {
        if (*abort_flag) return ~0u;
        if (clock64() - t0 > (1ll << 31)) {
            atomicOr(&scns[sc].clk->status, 2);
            *abort_flag = 1u;
            return ~0u;
        }
        __nanosleep(64);
    }
    return q;
}

/* thread 0 after an item of scenario sc: count it; true when it was the
 * scenario's last of the iteration */
__device__ __noinline__ bool count_item(const Scn32* __restrict__ scns, int nscn, int sc, Ctl32* ctl) {
    unsigned* cnt = reinterpret_cast<unsigned*>(reinterpret_cast<int*>(ctl + 1) + nscn);
    __threadfence(); /* the item's state and partial before its count */
    return atomicAdd(&cnt[sc], 1u) == (unsigned)scns[sc].nwork - 1u;
}

/* thread 0 after the scenario's reduction: release its next iteration */
__device__ __noinline__ void release_scenario(int nscn, int sc, int iterations_done, Ctl32* ctl) {
    int* done = reinterpret_cast<int*>(ctl + 1);
    unsigned* cnt = reinterpret_cast<unsigned*>(done + nscn);
    cnt[sc] = 0u;
    __threadfence();
    st_release_gpu(&done[sc], iterations_done);
}

/* niter iterations of the scenarios of one feature class.  Every CTA takes
 * queue tickets q = 0, 1, ...: ticket q is work item q % nwork of iteration
 * q / nwork.  Before an item of iteration it starts, its scenario must have
 * completed iteration it-1 in this launch (done[s] >= it).  The tickets a
 * scenario waits for were all handed out earlier to CTAs that are running
 * (the launch is cooperative: every CTA is resident), so the waits end; they
 * are bounded all the same (about 2^31 cycles), after which the CTA sets the
 * abort flag and the scenario's timeout bit, and every CTA leaves.  The CTA
 * that finishes a scenario's last item of an iteration reduces the
 * scenario's partials in a fixed order, advances its clock and releases
 * done[s] = it + 1.  done and cnt follow the control block, nscn ints each. */
template <bool CLS, bool RW, bool LAKE, bool SRC>
__global__ void __launch_bounds__(NT, 4) k32_persist(const Scn32* __restrict__ scns, int nscn,
                                                     const int4* __restrict__ work, int nwork, int niter,
                                                     Part32* __restrict__ part, Ctl32* ctl) {
    /* aligned by a byte offset from the shared array itself, so that the
     * compiler keeps the shared address space (shared loads, not generic) */
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SmemM& S = *reinterpret_cast<SmemM*>(smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u));
    if (threadIdx.x == 0) {
        for (int k = 0; k < NS; k++) mbar_init(&S.bar[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    unsigned gb = 0; /* staged blocks used so far by this CTA */
    if (threadIdx.x == 0) S.qn = atomicAdd(&ctl->next, 1u);
    for (;;) {
        if (threadIdx.x == 0) S.q = wait_ticket(S.qn, scns, work, nwork, niter, ctl);
        __syncthreads();
        /* read through a shuffle from lane 0: the compiler then knows the
         * ticket, the item and the scenario's fields are uniform across the
         * warp and keeps them in uniform registers, leaving the 128 per
         * thread to the marching windows */
        const unsigned q = __shfl_sync(0xffffffffu, S.q, 0);
        if (q == ~0u) break;
        if (threadIdx.x == 0) S.qn = atomicAdd(&ctl->next, 1u); /* the next ticket, drawn while this item runs */
        const int4 w = work[q % (unsigned)nwork];
        /* the previous iteration's state was written by other CTAs with
         * generic stores; this item reads it with TMA (the async proxy) */
        asm volatile("fence.proxy.async.global;" ::: "memory");
        if (!march_item<CLS, RW, LAKE, SRC>(S, scns[w.x], w, part, gb)) {
            if (threadIdx.x == 0) ctl->abort = 1u;
            break;
        }
        if (threadIdx.x == 0) S.last = count_item(scns, nscn, w.x, ctl);
        __syncthreads();
        if (__shfl_sync(0xffffffffu, S.last, 0)) {
            __threadfence();
            finalize_scn(scns[w.x], part, S.red, S.redf);
            if (threadIdx.x == 0) release_scenario(nscn, w.x, (int)(q / (unsigned)nwork) + 1, ctl);
        }
        __syncthreads();
    }
}

/* first slot of every scenario from its clock (t, s_max, t_end) */
__global__ void k32_prime(const Scn32* __restrict__ scns, int nscn) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nscn) return;
    volatile Clock32* clk = scns[s].clk;
    clk->done = 0;
    prepare_slot32(scns[s], clk, clk->t, clk->t_end, clk->s_max);
}

/* volume = sum of (h - kc) over active cells, and the CFL face speed of the
 * current state (the rule of k32_step), for one scenario (one block, fixed
 * order) */
/* Volume (depth minus its Kahan compensation, over active cells) and the
 * CFL face-speed sum of a scenario's current state: rows spread over up to
 * kVolBlocks blocks (columns over the threads, coalesced), partials reduced
 * in a fixed order by one block. */
constexpr int kVolBlocks = 1024;
struct VolPart {
    double vol;
    float sx, sy;
};

__device__ __forceinline__ void block_reduce_vol(double& vol, float& sx, float& sy) {
    __shared__ double sv[32];
    __shared__ float smx[32], smy[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vol += __shfl_xor_sync(0xffffffffu, vol, o);
        sx = fmaxf(sx, __shfl_xor_sync(0xffffffffu, sx, o));
        sy = fmaxf(sy, __shfl_xor_sync(0xffffffffu, sy, o));
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        sv[w] = vol;
        smx[w] = sx;
        smy[w] = sy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < nw; k++) {
            vol += sv[k];
            sx = fmaxf(sx, smx[k]);
            sy = fmaxf(sy, smy[k]);
        }
    }
}

__global__ void __launch_bounds__(256) k32_volume_part(const Scn32* __restrict__ scns, int iscn,
                                                       VolPart* __restrict__ part) {
    const Scn32& P = scns[iscn];
    const int cur = P.clk->slot.cur;
    const float th = P.th;
    double vol = 0.0;
    float sx = 0.f, sy = 0.f;
    for (int r = blockIdx.x; r < P.R; r += gridDim.x) {
        for (int c = threadIdx.x; c < P.C; c += blockDim.x) {
            const size_t g = (size_t)(r + M_H) * P.P + (c + M_H);
            if (!is_act(P.z[g])) continue;
            const float hh = P.h[cur][g];
            vol += (double)hh - (double)P.kc[g];
            if (r > 0 && is_act(P.z[g - P.P])) {
                const float hm = 0.5f * (hh + P.h[cur][g - P.P]);
                const float q = P.qx[cur][g];
                if (hm >= th) sx = fmaxf(sx, (fabsf(q != 0.f ? q / hm : 0.f) + fsqrt(P.g * hm)) * P.rdx);
            }
            if (c > 0 && is_act(P.z[g - 1])) {
                const float hn = 0.5f * (hh + P.h[cur][g - 1]);
                const float q = P.qy[cur][g];
                if (hn >= th) sy = fmaxf(sy, (fabsf(q != 0.f ? q / hn : 0.f) + fsqrt(P.g * hn)) * P.rdy);
            }
        }
    }
    block_reduce_vol(vol, sx, sy);
    if (threadIdx.x == 0) part[blockIdx.x] = VolPart{vol, sx, sy};
}

__global__ void __launch_bounds__(1024) k32_volume_fin(const Scn32* __restrict__ scns, int iscn,
                                                       const VolPart* __restrict__ part, int n, double* out) {
    const Scn32& P = scns[iscn];
    double vol = 0.0;
    float sx = 0.f, sy = 0.f;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        vol += part[k].vol;
        sx = fmaxf(sx, part[k].sx);
        sy = fmaxf(sy, part[k].sy);
    }
    block_reduce_vol(vol, sx, sy);
    if (threadIdx.x == 0) {
        out[0] = vol * P.area;
        out[1] = (double)sx + (double)sy;
    }
}

/* Boundary-discharge sample of an FP32 scenario (couple_BC_efdc,
 * SW2D-EFDC.cu:728-1067, with the argument swap of its call at :4909): one
 * thread per face (raster cell r * C + c, side 0 north / 1 south / 2 east /
 * 3 west), the cross-face velocity uua (north, south) or vva (east, west) of
 * the cell from the current state widened to binary64, inflow to the lake
 * only; the FP64 path's k_couple rule on the FP32 state. */
__device__ __forceinline__ double face_u32(const Scn32& P, const float* h, const float* q, int r, int c, double th) {
    const size_t i = (size_t)(r + M_H) * P.P + (c + M_H);
    double hm;
    if (r == 0) hm = (double)h[i];
    else if (r == P.R) hm = (double)h[i - P.P];
    else hm = 0.5 * ((double)h[i] + (double)h[i - P.P]);
    return hm >= th ? (double)q[i] / hm : 0.0;
}
__device__ __forceinline__ double face_v32(const Scn32& P, const float* h, const float* q, int r, int c, double th) {
    const size_t i = (size_t)(r + M_H) * P.P + (c + M_H);
    double hn;
    if (c == 0) hn = (double)h[i];
    else if (c == P.C) hn = (double)h[i - 1];
    else hn = 0.5 * ((double)h[i] + (double)h[i - 1]);
    return hn >= th ? (double)q[i] / hn : 0.0;
}

__global__ void k32_couple(const Scn32* __restrict__ scn, int nfaces, const int* __restrict__ faces, int lagged,
                           int initial, double th, double* __restrict__ vel_prev, double* __restrict__ qout) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nfaces) return;
    const Scn32& P = *scn;
    const int cur = P.clk->slot.cur;
    const float* h = P.h[cur];
    const float* qx = P.qx[cur];
    const float* qy = P.qy[cur];
    const int cell = faces[2 * k], side = faces[2 * k + 1];
    const int r = cell / P.C, c = cell - r * P.C;
    double vnow;
    if (side <= 1)
        vnow = (c > 0) ? 0.250 * (face_u32(P, h, qx, r, c, th) + face_u32(P, h, qx, r + 1, c, th) +
                                  face_u32(P, h, qx, r, c - 1, th) + face_u32(P, h, qx, r + 1, c - 1, th))
                       : 0.50 * (face_u32(P, h, qx, r, c, th) + face_u32(P, h, qx, r + 1, c, th));
    else
        vnow = (r > 0) ? 0.250 * (face_v32(P, h, qy, r, c, th) + face_v32(P, h, qy, r, c + 1, th) +
                                  face_v32(P, h, qy, r - 1, c, th) + face_v32(P, h, qy, r - 1, c + 1, th))
                       : 0.50 * (face_v32(P, h, qy, r, c, th) + face_v32(P, h, qy, r, c + 1, th));
    const double v = initial ? 0.0 : (lagged ? vel_prev[k] : vnow);
    const double hh = (double)h[(size_t)(r + M_H) * P.P + (c + M_H)];
    double out;
    switch (side) {
    case 1: out = (v < 0) ? -v * hh * P.dxd : 0.00; break; /* south */
    case 0: out = (v > 0) ? v * hh * P.dxd : 0.00; break;  /* north */
    case 2: out = (v < 0) ? -v * hh * P.dyd : 0.00; break; /* east */
    default: out = (v > 0) ? v * hh * P.dyd : 0.00; break; /* west */
    }
    qout[k] = out;
    vel_prev[k] = vnow;
}

void fp32_launch_couple(const Scn32* d_scn_one, int nfaces, const int* faces, int lagged, int initial, double th,
                        double* vel_prev, double* q, cudaStream_t s) {
    if (nfaces > 0)
        k32_couple<<<(nfaces + 127) / 128, 128, 0, s>>>(d_scn_one, nfaces, faces, lagged, initial, th, vel_prev, q);
}

size_t fp32_volume_scratch_bytes() { return 32 + kVolBlocks * sizeof(VolPart); }

typedef void (*PersistFn)(const Scn32*, int, const int4*, int, int, Part32*, Ctl32*);
static const PersistFn kPersist[T32_NCLASS] = {
    k32_persist<false, false, false, false>, k32_persist<true, false, false, false>,
    k32_persist<false, true, false, false>,  k32_persist<true, true, false, false>,
    k32_persist<false, false, true, false>,  k32_persist<true, false, true, false>,
    k32_persist<false, true, true, false>,   k32_persist<true, true, true, false>,
    k32_persist<false, false, false, true>,  k32_persist<true, false, false, true>,
    k32_persist<false, true, false, true>,   k32_persist<true, true, false, true>,
    k32_persist<false, false, true, true>,   k32_persist<true, false, true, true>,
    k32_persist<false, true, true, true>,    k32_persist<true, true, true, true>,
};

int fp32_feature_class(const Scn32& d) {
    return (d.cls ? 1 : 0) | (d.rainw ? 2 : 0) | (d.ledger_cells ? 4 : 0) | (d.nsrc > 0 ? 8 : 0);
}

int fp32_configure_kernels() {
    for (int k = 0; k < T32_NCLASS; k++) {
        cudaError_t e = cudaFuncSetAttribute(kPersist[k], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)fp32_smem_bytes_variant(k));
        if (e != cudaSuccess) return -1;
    }
    return 0;
}

int fp32_blocks_per_sm(int k) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kPersist[k], NT, fp32_smem_bytes_variant(k)) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t fp32_launch_chunk(const Scn32* d_scn, int nscn, const int4* d_work, const int* class_first,
                              const int* class_n, Part32* d_part, void* d_ctl, int niter, const int* grid,
                              cudaStream_t s) {
    for (int k = 0; k < T32_NCLASS; k++) {
        if (class_n[k] <= 0) continue;
        cudaError_t e = cudaMemsetAsync(d_ctl, 0, fp32_ctl_bytes(nscn), s);
        if (e != cudaSuccess) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid[k]);
        cfg.blockDim = dim3(NT);
        cfg.dynamicSmemBytes = fp32_smem_bytes_variant(k);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative; /* every CTA resident: the dataflow waits end */
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, kPersist[k], d_scn, nscn, d_work + class_first[k], class_n[k], niter, d_part,
                               static_cast<Ctl32*>(d_ctl));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void fp32_launch_prime(const Scn32* d_scn, int nscn, cudaStream_t s) {
    k32_prime<<<(nscn + 127) / 128, 128, 0, s>>>(d_scn, nscn);
}

void fp32_launch_volume(const Scn32* d_scn, int iscn, const Scn32& host_scn, double* d_out, cudaStream_t s) {
    const int nb = std::max(1, std::min(host_scn.R, kVolBlocks));
    VolPart* part = reinterpret_cast<VolPart*>(reinterpret_cast<char*>(d_out) + 32);
    k32_volume_part<<<nb, 256, 0, s>>>(d_scn, iscn, part);
    k32_volume_fin<<<1, 1024, 0, s>>>(d_scn, iscn, part, nb, d_out);
}

} // namespace sw2d
