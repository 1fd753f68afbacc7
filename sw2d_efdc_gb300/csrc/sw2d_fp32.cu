/* FP32 precision form of the SW2D step on sm_103a: one row-marching kernel
 * per iteration.
 *
 * A work item is a 224-column strip x `seg` rows of one scenario, taken by a
 * CTA of four warps.  Thread 0 streams the strip's rows (232 columns with a
 * 4-cell halo) of depth, bed offset and x/y discharges into a three-block
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
 * every field once from HBM and writes it once.  A second, tiny kernel
 * reduces each scenario's work-item partials in a fixed order and prepares
 * the scenario's next iteration (CFL length, rain).
 *
 * Arithmetic is binary32 except the clock, the ledger and the CFL length
 * (binary64).  Gravity uses (h_e - h_w) + (z_e - z_w) with bed offsets from
 * the tile datum, so no large elevations are added to small depths.
 */
#include "sw2d_fp32.h"

#include <math.h>
#include <stddef.h>

namespace sw2d {

#define NW M_NW
#define BW M_BW
#define RB M_RB
#define NS M_NS
#define NT M_NT

struct SmemM {
    alignas(128) float stage[NS][4][RB][BW]; /* h, z, qx, qy */
    unsigned long long bar[NS];
    float ntab[T32_MAXCLASS];
    float dd[9];
    double red[NW][4];
    float redf[NW][2];
};
static_assert(offsetof(SmemM, stage) % 128 == 0, "TMA alignment");
static_assert((RB * BW * 4) % 128 == 0, "each staged array is whole 128-byte lines");
static_assert((BW * 4) % 16 == 0, "TMA inner extent must be a multiple of 16 bytes");

size_t fp32_smem_bytes() { return sizeof(SmemM) + 128; }

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

/* binary32 math from the hardware approximations (a few ulp; the precision
 * form does not need IEEE rounding) */
__device__ __forceinline__ float frcp(float x) { return __frcp_rn(x); }
__device__ __forceinline__ float fsqrt(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }
__device__ __forceinline__ float rpow_manning_f32(float hm) { return __powf(hm, -1.3333330f); } /* hm^-1.333333 */

__device__ __forceinline__ bool is_act(float z) { return z == z; } /* NaN bed offset = inactive */

/* value of the neighbouring column on the left / right for the lane's two
 * columns (2l, 2l+1) */
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
__device__ __forceinline__ float comp(float2 v, int k) { return k ? v.y : v.x; }
__device__ __forceinline__ void setc(float2& v, int k, float x) {
    if (k) v.y = x;
    else v.x = x;
}

/* Upwind donor-cell transport across the edge between two faces of the same
 * orientation (the reference's umr/uml, umu/umd, vnr/vnl, vnu/vnd terms,
 * SW2D-EFDC.cu:171-189, :288-306): with a = half the mean of the two face
 * velocities, a (q1 + q0) + |a| (q0 - q1), q0 on the upstream-indexed face.
 * Each edge is shared by the two faces it separates, so it is computed once. */
__device__ __forceinline__ float edge_term(float w_quarter, float q0, float q1) {
    return w_quarter * (q1 + q0) + fabsf(w_quarter) * (q0 - q1);
}

struct FaceIn {
    float hw, he, zw, ze;  /* the two cells (w: north / west, e: south / east) */
    float q0, u0, vt;      /* old discharge, face velocity, cross velocity at the face */
    float along, across;   /* convection differences (edge terms, already scaled) */
    float gdt2n;           /* g * dt2 / spacing along the normal */
    float gn2;             /* g * n_face^2 */
};

/* One face of the reference's flux (SW2D-EFDC.cu:110-202 x, :228-319 y) in
 * binary32, evaluated without branches so that a lane's four faces
 * interleave: the weir / dry-bed / momentum results are selected by the
 * reference's conditions. */
__device__ __forceinline__ float face_flux(const FaceIn& f, float th, float g, float hdt2) {
    const float he = f.he, hw = f.hw, ze = f.ze, zw = f.zw;
    const bool act = is_act(ze) && is_act(zw);
    const bool wet = (hw > th) || (he > th);
    const float hhe = he + ze, hhw = hw + zw;
    const float hhep = he - th, hhwp = hw - th;
    const bool d1a = hhe < zw, d1b = hhw < ze;
    const bool d2 = hhep * hhwp < 0.f;
    /* dry bed 1: free overfall from the higher cell (:129-144) */
    const float hup = d1a ? hw : he;
    const float fw = (hup > th) ? (d1a ? 0.5440f : -0.544f) * hup * fsqrt(g * hup) : 0.f;
    /* dry bed 2 (:148-157) */
    const float hh3 = fmaxf(hhe, hhw) - fmaxf(ze, zw);
    const float fd = ((he > 0.f) || (hw > 0.f)) ? -copysignf(0.350f, hhep - hhwp) * hh3 * fsqrt(2.f * g * hh3) : 0.f;
    /* momentum: gravity, convection, semi-implicit Manning friction (:165-202) */
    const float hm = 0.5f * (he + hw);
    const float grav = f.gdt2n * hm * ((he - hw) + (ze - zw));
    const float sq = fsqrt(f.u0 * f.u0 + f.vt * f.vt);
    const float ram = (hm > th) ? f.gn2 * sq * rpow_manning_f32(hm) : 0.f;
    const float a = hdt2 * ram;
    const float fm = ((1.f - a) * f.q0 - f.along - f.across - grav) * frcp(1.f + a);
    const float F = (d1a || d1b) ? fw : (d2 ? fd : fm);
    return (act && wet) ? F : 0.f;
}

/* ---------------- the row-marching step ---------------------------------- */

__global__ void __launch_bounds__(NT, 4) k32_march(const Scn32* __restrict__ scns, const int4* __restrict__ work,
                                                   Part32* __restrict__ part) {
    extern __shared__ unsigned char smem_raw[];
    SmemM& S = *reinterpret_cast<SmemM*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int4 w = work[blockIdx.x];
    const Scn32& P = scns[w.x];
    Clock32* clk = P.clk;
    const Slot32 sl = clk->slot;
    if (!sl.active) {
        if (tid == 0) {
            Part32 zp = {};
            part[blockIdx.x] = zp;
        }
        return;
    }
    const int cur = sl.cur, nxt = cur ^ 1;
    const int R = P.R, C = P.C, Pp = P.P;
    const int strip = w.y, seg = w.z;
    const int c0 = strip * M_CW;             /* first output column of the strip */
    const int rs = seg * P.seg, re = min(rs + P.seg, R);
    const int Ls = rs - 3;                   /* first staged row */
    const int nblk = (re - rs + 6 + RB - 1) / RB;

    if ((smem_addr(&S.stage[0][0][0][0]) & 127u) != 0u) {
        if (tid == 0) atomicOr(&clk->status, 4);
        return;
    }
    if (tid == 0) {
        for (int k = 0; k < NS; k++) mbar_init(&S.bar[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid < T32_MAXCLASS) S.ntab[tid] = P.ntab[tid];
    if (tid < 9) {
        const int dy = tid / 3 - 1, dx = tid % 3 - 1;
        const int ny = seg + dy, nx = strip + dx;
        float d = 0.f;
        if (ny >= 0 && ny < P.tiles_y && nx >= 0 && nx < P.tiles_x)
            d = P.datum[ny * P.tiles_x + nx] - P.datum[seg * P.tiles_x + strip];
        S.dd[tid] = d;
    }
    __syncthreads();
    const unsigned blk_bytes = 4u * RB * BW * 4u;
    if (tid == 0) {
        for (int b = 0; b < NS && b < nblk; b++) {
            mbar_arrive_expect_tx(&S.bar[b], blk_bytes);
            const int y = Ls + b * RB + M_H; /* padded row of the block's first row */
            tma_load_2d(&S.stage[b][0][0][0], &P.tm_h[cur], c0, y, &S.bar[b]);
            tma_load_2d(&S.stage[b][1][0][0], &P.tm_z, c0, y, &S.bar[b]);
            tma_load_2d(&S.stage[b][2][0][0], &P.tm_qx[cur], c0, y, &S.bar[b]);
            tma_load_2d(&S.stage[b][3][0][0], &P.tm_qy[cur], c0, y, &S.bar[b]);
        }
    }

    /* lane geometry: staged columns sc, sc+1; global columns cg, cg+1 */
    const int sc = warp * M_SW + 2 * lane;
    const int cg = c0 - M_H + sc;
    const bool own0 = (lane >= 2 && lane < 30) && cg < C;
    const bool own1 = (lane >= 2 && lane < 30) && cg + 1 < C;
    const int creg0 = sc < M_H ? 0 : (sc >= M_H + M_CW ? 2 : 1);
    const int creg1 = sc + 1 < M_H ? 0 : (sc + 1 >= M_H + M_CW ? 2 : 1);
    /* datum shifts of the lane's two columns for rows above / inside / below the segment */
    const float dzt0 = S.dd[creg0], dzm0 = S.dd[3 + creg0], dzb0 = S.dd[6 + creg0];
    const float dzt1 = S.dd[creg1], dzm1 = S.dd[3 + creg1], dzb1 = S.dd[6 + creg1];
    const float th = P.th, gg = P.g, rdx = P.rdx, rdy = P.rdy;
    const float dt2 = sl.dt2, dt2dx = sl.dt2dx, dt2dy = sl.dt2dy, hdt2 = 0.5f * sl.dt2;
    const float gdx = gg * dt2dx, gdy = gg * dt2dy;
    const bool has_cls = P.cls != nullptr, has_rw = P.rainw != nullptr;
    const float n_uni = S.ntab[0], gn2_uni = gg * n_uni * n_uni;
    const bool col0_0 = (cg == 0), col0_1 = (cg + 1 == 0);

    /* register windows, slot = (row - Ls) & 3 */
    float2 H[4], Z[4], QX[4], QY[4], U[4], V[4], FX[4], FY[4];
    float2 HL[4], ZL[4], UL[4], VR[4], FYR[4], RW[4], NN[4], NL[4], EX[4], GY[4];
    int DRY[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        H[k] = Z[k] = QX[k] = QY[k] = U[k] = V[k] = FX[k] = FY[k] = make_float2(0.f, 0.f);
        HL[k] = ZL[k] = UL[k] = VR[k] = FYR[k] = NN[k] = NL[k] = EX[k] = GY[k] = make_float2(0.f, 0.f);
        RW[k] = make_float2(1.f, 1.f);
        DRY[k] = 0;
    }
    float clamp = 0.f, qout = 0.f, rainacc = 0.f, evc = 0.f, sxm = 0.f, sym = 0.f;

    for (int b = 0; b < nblk; b++) {
        const int st = b % NS;
        /* bounded wait for the block (about 2^31 cycles); the CTA agrees on
         * the outcome so that no warp is left waiting at a barrier */
        {
            const unsigned par = (unsigned)((b / NS) & 1);
            long long t0 = clock64();
            bool ok = true;
            while (!mbar_try_wait(&S.bar[st], par)) {
                if (clock64() - t0 > (1ll << 31)) {
                    ok = false;
                    break;
                }
            }
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(&clk->status, 2);
                return;
            }
        }
        const float* sh = &S.stage[st][0][0][0];
        const float* sz = &S.stage[st][1][0][0];
        const float* sqx = &S.stage[st][2][0][0];
        const float* sqy = &S.stage[st][3][0][0];
#pragma unroll
        for (int j = 0; j < RB; j++) {
            const int L = Ls + b * RB + j;
            const int s0 = j & 3, s1 = (j + 3) & 3, s2 = (j + 2) & 3, s3 = (j + 1) & 3; /* L, L-1, L-2, L-3 */
            /* ---- row L from the staged block ---- */
            H[s0] = *reinterpret_cast<const float2*>(sh + j * BW + sc);
            float2 zz = *reinterpret_cast<const float2*>(sz + j * BW + sc);
            zz.x += L < rs ? dzt0 : (L >= re ? dzb0 : dzm0);
            zz.y += L < rs ? dzt1 : (L >= re ? dzb1 : dzm1);
            Z[s0] = zz;
            QX[s0] = *reinterpret_cast<const float2*>(sqx + j * BW + sc);
            QY[s0] = *reinterpret_cast<const float2*>(sqy + j * BW + sc);
            const bool rowin = (L >= -M_H && L < R + M_H) && cg + M_H >= 0 && cg + M_H + 1 < Pp;
            const size_t gL = (size_t)(L + M_H) * Pp + (cg + M_H);
            if (has_cls) {
                float2 nn = make_float2(n_uni, n_uni);
                if (rowin) {
                    const uchar2 cc = *reinterpret_cast<const uchar2*>(P.cls + gL);
                    nn = make_float2(S.ntab[cc.x & 63], S.ntab[cc.y & 63]);
                }
                NN[s0] = nn;
                NL[s0] = left2(nn);
            }
            if (has_rw) RW[s0] = rowin ? *reinterpret_cast<const float2*>(P.rainw + gL) : make_float2(1.f, 1.f);
            HL[s0] = left2(H[s0]);
            ZL[s0] = left2(Z[s0]);
            /* ---- face velocities of row L and CFL face speeds of owned faces ---- */
            const bool rowown = (L >= rs && L < re);
#pragma unroll
            for (int k = 0; k < 2; k++) {
                const float hLk = comp(H[s0], k);
                const float hm = (L == R) ? comp(H[s1], k) : 0.5f * (hLk + comp(H[s1], k));
                const float u = (hm >= th) ? comp(QX[s0], k) * frcp(hm) : 0.f;
                setc(U[s0], k, u);
                const float hn = 0.5f * (hLk + comp(HL[s0], k));
                const float v = (hn >= th) ? comp(QY[s0], k) * frcp(hn) : 0.f;
                setc(V[s0], k, v);
                const bool own = (k ? own1 : own0) && rowown;
                const bool za = is_act(comp(Z[s0], k));
                const bool okx = own && hm >= th && za && is_act(comp(Z[s1], k));
                const bool oky = own && hn >= th && za && is_act(comp(ZL[s0], k));
                sxm = fmaxf(sxm, okx ? (fabsf(u) + fsqrt(gg * hm)) * rdx : 0.f);
                sym = fmaxf(sym, oky ? (fabsf(v) + fsqrt(gg * hn)) * rdy : 0.f);
            }
            UL[s0] = left2(U[s0]);
            VR[s0] = right2(V[s0]);
            /* ---- edge terms: along x between x faces L-1 and L, cross for y faces
             *      between rows L-1 and L, and the two edge kinds of row L-1 ---- */
            const float2 qxr = right2(QX[s1]), qyr = right2(QY[s1]);
            float2 EY, GX;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                setc(EX[s1], k, edge_term(0.25f * (comp(U[s0], k) + comp(U[s1], k)), comp(QX[s1], k), comp(QX[s0], k)));
                setc(GY[s1], k, edge_term(0.25f * (comp(U[s0], k) + comp(UL[s0], k)), comp(QY[s1], k), comp(QY[s0], k)));
                setc(EY, k, edge_term(0.25f * (comp(VR[s1], k) + comp(V[s1], k)), comp(QY[s1], k), comp(qyr, k)));
                setc(GX, k, edge_term(0.25f * (comp(VR[s1], k) + comp(VR[s2], k)), comp(QX[s1], k), comp(qxr, k)));
            }
            const float2 EYL = left2(EY), GXL = left2(GX);
            /* ---- face discharges of row L-1 ---- */
            const int rf = L - 1;
#pragma unroll
            for (int k = 0; k < 2; k++) {
                FaceIn fx;
                fx.hw = comp(H[s2], k);
                fx.he = comp(H[s1], k);
                fx.zw = comp(Z[s2], k);
                fx.ze = comp(Z[s1], k);
                fx.q0 = comp(QX[s1], k);
                fx.u0 = comp(U[s1], k);
                fx.vt = 0.25f * (comp(V[s1], k) + comp(V[s2], k) + comp(VR[s1], k) + comp(VR[s2], k));
                fx.along = dt2dx * (comp(EX[s1], k) - comp(EX[s2], k));
                fx.across = (k ? col0_1 : col0_0) ? 0.f : dt2dy * (comp(GX, k) - comp(GXL, k));
                fx.gdt2n = gdx;
                if (has_cls) {
                    const float nf = 0.5f * (comp(NN[s1], k) + comp(NN[s2], k));
                    fx.gn2 = gg * nf * nf;
                } else {
                    fx.gn2 = gn2_uni;
                }
                float F = face_flux(fx, th, gg, hdt2);
                if (rf == R) { /* south edge: free overfall when open (SW2D-EFDC.cu:131 law) */
                    const float hw = fx.hw;
                    F = (P.outflow_south && is_act(fx.zw) && hw > th) ? 0.5440f * hw * fsqrt(gg * hw) : 0.f;
                }
                setc(FX[s1], k, F);
                FaceIn fy;
                fy.hw = comp(HL[s1], k);
                fy.he = comp(H[s1], k);
                fy.zw = comp(ZL[s1], k);
                fy.ze = comp(Z[s1], k);
                fy.q0 = comp(QY[s1], k);
                fy.u0 = comp(V[s1], k);
                fy.vt = 0.25f * (comp(U[s1], k) + comp(U[s0], k) + comp(UL[s1], k) + comp(UL[s0], k));
                fy.along = dt2dy * (comp(EY, k) - comp(EYL, k));
                fy.across = (rf == 0) ? 0.f : dt2dx * (comp(GY[s1], k) - comp(GY[s2], k));
                fy.gdt2n = gdy;
                if (has_cls) {
                    const float nf = 0.5f * (comp(NN[s1], k) + comp(NL[s1], k));
                    fy.gn2 = gg * nf * nf;
                } else {
                    fy.gn2 = gn2_uni;
                }
                setc(FY[s1], k, face_flux(fy, th, gg, hdt2));
            }
            /* ---- provisional depth of row L-2 -> dry flags ---- */
            FYR[s2] = right2(FY[s2]);
            {
                int dry = 0;
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    const float ho = comp(H[s2], k);
                    const bool lake = ho > P.ev_wl_min;
                    const float pct = lake ? P.pct_lake : P.pct_land;
                    const float ev = lake ? sl.ev1 : 0.f;
                    const float hs = ho - dt2 * ((comp(FX[s1], k) - comp(FX[s2], k)) * rdx +
                                                 (comp(FYR[s2], k) - comp(FY[s2], k)) * rdy -
                                                 sl.rr1 * comp(RW[s2], k) * pct + ev);
                    dry |= (is_act(comp(Z[s2], k)) && hs < th) ? (1 << k) : 0;
                }
                DRY[s2] = dry;
            }
            /* ---- final depth of row L-3 ---- */
            {
                const int r = L - 3;
                const int dc = DRY[s3], dN = DRY[s0], dS = DRY[s2];
                const int dW = leftbits(dc), dE = rightbits(dc);
                if (r >= rs && r < re && (own0 || own1)) {
                    const size_t g = (size_t)(r + M_H) * Pp + (cg + M_H);
                    const float2 kcv = own1 ? *reinterpret_cast<const float2*>(P.kc + g) : make_float2(P.kc[g], 0.f);
                    float2 hout, kout, fNo, fWo, fSo;
#pragma unroll
                    for (int k = 0; k < 2; k++) {
                        float fN = comp(FX[s3], k), fS = comp(FX[s2], k), fW = comp(FY[s3], k), fE = comp(FYR[s3], k);
                        const int bc = (dc >> k) & 1;
                        fN = ((fN > 0.f && ((dN >> k) & 1)) || (fN < 0.f && bc)) ? 0.f : fN;
                        fS = ((fS > 0.f && bc) || (fS < 0.f && ((dS >> k) & 1))) ? 0.f : fS;
                        fW = ((fW > 0.f && ((dW >> k) & 1)) || (fW < 0.f && bc)) ? 0.f : fW;
                        fE = ((fE > 0.f && bc) || (fE < 0.f && ((dE >> k) & 1))) ? 0.f : fE;
                        const bool own = k ? own1 : own0;
                        const bool act = is_act(comp(Z[s3], k));
                        const float ho = comp(H[s3], k);
                        const float wgt = comp(RW[s3], k);
                        const bool lake = ho > P.ev_wl_min;
                        const float pct = lake ? P.pct_lake : P.pct_land;
                        const float ev = lake ? sl.ev2 : 0.f;
                        const float dh = -dt2 * ((fS - fN) * rdx + (fE - fW) * rdy - sl.rr2 * wgt * pct + ev);
                        /* Kahan: the increment is small against the depth */
                        const float y = dh - comp(kcv, k);
                        const float t = ho + y;
                        float kc = (t - ho) - y;
                        float hn = t;
                        if (own && act) {
                            clamp += hn < 0.f ? -hn : 0.f;
                            if (P.ledger_cells) {
                                rainacc += wgt * pct;
                                evc += lake ? 1.f : 0.f;
                            }
                            if (r == R - 1) qout += fS;
                        }
                        kc = (act && hn >= 0.f) ? kc : 0.f;
                        hn = act ? fmaxf(hn, 0.f) : 0.f;
                        setc(hout, k, hn);
                        setc(kout, k, kc);
                        setc(fNo, k, fN);
                        setc(fWo, k, fW);
                        setc(fSo, k, fS);
                    }
                    if (own0 && own1) {
                        *reinterpret_cast<float2*>(P.h[nxt] + g) = hout;
                        *reinterpret_cast<float2*>(P.kc + g) = kout;
                        *reinterpret_cast<float2*>(P.qx[nxt] + g) = fNo;
                        *reinterpret_cast<float2*>(P.qy[nxt] + g) = fWo;
                        if (r == R - 1) *reinterpret_cast<float2*>(P.qx[nxt] + g + Pp) = fSo;
                    } else {
                        P.h[nxt][g] = hout.x;
                        P.kc[g] = kout.x;
                        P.qx[nxt][g] = fNo.x;
                        P.qy[nxt][g] = fWo.x;
                        if (r == R - 1) P.qx[nxt][g + Pp] = fSo.x;
                    }
                }
            }
        }
        __syncthreads(); /* every warp is done with block b */
        if (tid == 0 && b + NS < nblk) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive_expect_tx(&S.bar[st], blk_bytes);
            const int y = Ls + (b + NS) * RB + M_H;
            tma_load_2d(&S.stage[st][0][0][0], &P.tm_h[cur], c0, y, &S.bar[st]);
            tma_load_2d(&S.stage[st][1][0][0], &P.tm_z, c0, y, &S.bar[st]);
            tma_load_2d(&S.stage[st][2][0][0], &P.tm_qx[cur], c0, y, &S.bar[st]);
            tma_load_2d(&S.stage[st][3][0][0], &P.tm_qy[cur], c0, y, &S.bar[st]);
        }
    }

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
        pr.sx = mx;
        pr.sy = my;
        part[blockIdx.x] = pr;
    }
}

/* ---------------- per-scenario finalize ---------------------------------- */

__device__ double series_at32(const double* v, int n, double dts, double time, int mode) {
    int it;
    if (mode == 0) {
        if (time <= 1.00) return v[0] * time;
        it = (int)(time / dts);
        if (it + 1 > n) it = n;
        return v[it] + (v[it + 1] - v[it]) / (dts * (time - dts * (it)));
    } else if (mode == 1) {
        it = (int)(time / dts);
        if (it + 1 > n) it = n;
        return v[it] + (v[it + 1] - v[it]) * ((time - dts * (it)) / dts);
    }
    it = (int)(time / dts);
    if (it > n) it = n;
    return v[it];
}

__device__ void prepare_slot32(const Scn32& P, Clock32* clk) {
    const double t = clk->t;
    double dt2, tm;
    int active;
    if (P.dt_mode == 0) {
        const double dt = P.dt_fixed;
        active = (t + dt <= clk->t_end);
        dt2 = (double)(float)(2.0 * dt);
        tm = t + dt;
    } else {
        active = (t < clk->t_end);
        dt2 = clk->s_max > 0 ? fmin(P.dt_max, P.cfl / clk->s_max) : P.dt_max;
        dt2 = (double)(float)dt2;
        if (t + dt2 > clk->t_end) dt2 = clk->t_end - t;
        tm = t + 0.5 * dt2;
    }
    Slot32& s = clk->slot;
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
    clk->dt2 = dt2;
    if (!active) clk->done = 1;
}

/* one warp per scenario: fixed-order sum of its tile partials */
__global__ void k32_finalize(const Scn32* __restrict__ scns, int nscn, const Part32* __restrict__ part) {
    const int s = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (s >= nscn) return;
    const Scn32& P = scns[s];
    Clock32* clk = P.clk;
    if (!clk->slot.active) return;
    double clamp = 0, qout = 0, rain = 0, evc = 0;
    float sx = 0.f, sy = 0.f;
    for (int k = lane; k < P.nwork; k += 32) {
        const Part32& q = part[P.first_work + k];
        clamp += q.clamp;
        qout += q.qout;
        rain += q.rain;
        evc += q.evap;
        sx = fmaxf(sx, q.sx);
        sy = fmaxf(sy, q.sy);
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
    if (lane != 0) return;
    const Slot32 sl = clk->slot;
    const double dt2 = clk->dt2;
    const double area = P.area;
    const double rain_sum = P.ledger_cells ? rain : P.rain_static;
    clk->rain_in += dt2 * (double)sl.rr2 * rain_sum * area;
    clk->evap_out += dt2 * (double)sl.ev2 * evc * area;
    clk->clamp_gain += clamp * area;
    clk->q_out = qout * P.dyd;
    clk->outflow += dt2 * clk->q_out;
    /* the CFL speed of the state this iteration started from */
    clk->s_max = (double)sx + (double)sy;
    if (!isfinite(clk->s_max) || !isfinite(qout)) clk->status |= 1;
    clk->t = clk->t + dt2;
    clk->iters += 1;
    clk->slot.cur = sl.cur ^ 1;
    if (P.outlet) {
        const long long k = clk->outlet_n % P.outlet_cap;
        P.outlet[2 * k] = clk->t;
        P.outlet[2 * k + 1] = clk->q_out;
        clk->outlet_n += 1;
    }
    prepare_slot32(P, clk);
}

/* first slot of every scenario from its clock (t, s_max, t_end) */
__global__ void k32_prime(const Scn32* __restrict__ scns, int nscn) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nscn) return;
    Clock32* clk = scns[s].clk;
    clk->done = 0;
    prepare_slot32(scns[s], clk);
}

/* volume = sum of (h - kc) over active cells, and the CFL face speed of the
 * current state (the rule of k32_step), for one scenario (one block, fixed
 * order) */
__global__ void k32_volume(const Scn32* __restrict__ scns, int iscn, double* out) {
    const Scn32& P = scns[iscn];
    const int cur = P.clk->slot.cur;
    const float th = P.th;
    double vol = 0.0;
    float sx = 0.f, sy = 0.f;
    for (long long k = threadIdx.x; k < (long long)P.R * P.C; k += blockDim.x) {
        const int r = (int)(k / P.C), c = (int)(k % P.C);
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
    __shared__ double sv[1024];
    __shared__ float smx[1024], smy[1024];
    sv[threadIdx.x] = vol;
    smx[threadIdx.x] = sx;
    smy[threadIdx.x] = sy;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sv[threadIdx.x] += sv[threadIdx.x + o];
            smx[threadIdx.x] = fmaxf(smx[threadIdx.x], smx[threadIdx.x + o]);
            smy[threadIdx.x] = fmaxf(smy[threadIdx.x], smy[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sv[0] * P.area;
        out[1] = (double)smx[0] + (double)smy[0];
    }
}

int fp32_configure_kernels() {
    cudaError_t e = cudaFuncSetAttribute(k32_march, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fp32_smem_bytes());
    return e == cudaSuccess ? 0 : -1;
}

void fp32_launch_iteration(const Scn32* d_scn, int nscn, const int4* d_work, int nwork, Part32* d_part,
                           cudaStream_t s) {
    if (nwork > 0) k32_march<<<nwork, NT, fp32_smem_bytes(), s>>>(d_scn, d_work, d_part);
    k32_finalize<<<(nscn + 3) / 4, 128, 0, s>>>(d_scn, nscn, d_part);
}

void fp32_launch_prime(const Scn32* d_scn, int nscn, cudaStream_t s) {
    k32_prime<<<(nscn + 127) / 128, 128, 0, s>>>(d_scn, nscn);
}

void fp32_launch_volume(const Scn32* d_scn, int iscn, const Scn32& host_scn, double* d_out, cudaStream_t s) {
    (void)host_scn;
    k32_volume<<<1, 1024, 0, s>>>(d_scn, iscn, d_out);
}

} // namespace sw2d
