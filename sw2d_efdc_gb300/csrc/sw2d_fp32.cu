/* FP32 precision form of the SW2D step on sm_103a: one fused kernel per
 * iteration.
 *
 * Each CTA owns a 64 x 32 tile of one scenario.  Thread 0 stages the tile
 * with a 4-cell halo (72 x 40) of depth, bed offset, x/y discharges and the
 * info byte into shared memory with five 2-D TMA loads
 * (cp.async.bulk.tensor, one mbarrier); then, all in shared memory:
 *   1. face velocities uu1 = qx/hm, vv1 = qy/hn        (hm_hn, uu1_vv1: SW2D-EFDC.cu:362-452)
 *   2. new x and y face discharges                        (flux: :97-353)
 *   3. provisional depth at t on the tile and a 1-cell ring -> "dry" bytes
 *                                                         (continuity :602-664)
 *   4. outward faces of dry cells closed                   (treat_error :695-725, per face)
 *      final depth at t+dt with a Kahan-compensated increment, written
 *      with the tile's north/west faces; block reductions of the CFL speed
 *      and of the ledger terms.
 * The halo is recomputed instead of exchanged, so an iteration reads every
 * field once from HBM and writes it once (neighbouring tiles' halo reads hit
 * L2).  A second, tiny kernel reduces each scenario's tile partials in a
 * fixed order and prepares the scenario's next iteration (CFL length, rain).
 *
 * Arithmetic is binary32 except the clock, the ledger and the CFL length
 * (binary64).  Gravity uses (h_e - h_w) + (z_e - z_w) with bed offsets from
 * the tile datum, so no large elevations are added to small depths.
 */
#include "sw2d_fp32.h"

#include <math.h>
#include <stddef.h>

namespace sw2d {

#define TC T32_TC
#define TR T32_TR
#define LW T32_LW
#define LH T32_LH
#define LWB T32_LWB
#define NT T32_NT

/* staged region: local row lr in [0, 40), col lc in [0, 72); global row r0 - 4 + lr */
#define U_W 68 /* uu1 rows [2, 39), cols [2, 70) */
#define U_H 37
#define V_W 69 /* vv1 rows [2, 38), cols [2, 71) */
#define V_H 36
#define D_W 66 /* dry rows [3, 37), cols [3, 69) */
#define D_H 34
#define FX_W 66 /* x faces rows [3, 38), cols [3, 69) */
#define FX_H 35
#define FY_W 67 /* y faces rows [3, 37), cols [3, 70) */
#define FY_H 34

/* TMA tensor copies need 128-byte aligned shared destinations: the five
 * staged arrays come first, each a multiple of 128 bytes long. */
struct Smem32 {
    alignas(128) float h[LH * LW];
    alignas(128) float z[LH * LW];
    alignas(128) float qx[LH * LW];
    alignas(128) float qy[LH * LW];
    alignas(128) uint8_t info[LH * LWB];
    alignas(128) float u[U_H * U_W];
    float v[V_H * V_W];
    uint8_t dry[D_H * D_W];
    float ntab[T32_MAXCLASS];
    float dd[9];
    double red[8][4];
    float redf[8][2];
    unsigned long long bar;
};
static_assert(offsetof(Smem32, h) % 128 == 0 && offsetof(Smem32, z) % 128 == 0, "TMA alignment");
static_assert(offsetof(Smem32, qx) % 128 == 0 && offsetof(Smem32, qy) % 128 == 0, "TMA alignment");
static_assert(offsetof(Smem32, info) % 128 == 0, "TMA alignment");
static_assert(offsetof(Smem32, bar) % 8 == 0, "mbarrier alignment");
static_assert((LH * LW * 4) % 128 == 0 && (LH * LWB) % 128 == 0, "staged arrays are whole 128-byte lines");

size_t fp32_smem_bytes() { return sizeof(Smem32) + 128; }

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

/* Wait for the staged tile with a bounded spin: about 2^31 clock cycles (~1 s).
 * On timeout the scenario's status records it and the CTA gives up. */
__device__ __forceinline__ bool wait_tile(unsigned long long* bar, Clock32* clk) {
    long long t0 = clock64();
    while (!mbar_try_wait(bar, 0)) {
        if (clock64() - t0 > (1ll << 31)) {
            if (threadIdx.x == 0) atomicOr(&clk->status, 2);
            /* second bounded wait for the copies already in flight */
            long long t1 = clock64();
            while (!mbar_try_wait(bar, 0) && clock64() - t1 < (1ll << 31)) {
            }
            return false;
        }
    }
    return true;
}

/* ---------------- device helpers ---------------------------------------- */

__device__ __forceinline__ float rpow_manning_f32(float hm) {
    /* hm^-1.3333330 from the hardware log2/exp2 (relative error ~1e-6) */
    return __powf(hm, -1.3333330f);
}

/* binary32 square root and quotient from the hardware reciprocal
 * approximations (a few ulp; the precision form does not need IEEE rounding) */
__device__ __forceinline__ float fsqrt(float x) { return x > 0.f ? x * rsqrtf(x) : 0.f; }
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }

/* x face between staged cells (lr-1, lc) "w" and (lr, lc) "e" */
__device__ __forceinline__ float flux_x32(const Smem32& S, const Scn32& P, const Slot32& sl, int lr, int lc,
                                          int r, int c) {
    const int e = lr * LW + lc, w = e - LW;
    const float th = P.th, gg = P.g;
    const float he = S.h[e], hw = S.h[w];
    const uint8_t ie = S.info[lr * LWB + lc], iw = S.info[(lr - 1) * LWB + lc];
    if (r == P.R && P.outflow_south) {
        if ((iw & SW2D_I_ACTIVE) && hw > th) return 0.5440f * hw * fsqrt(gg * hw);
        return 0.f;
    }
    if (!(ie & iw & SW2D_I_ACTIVE)) return 0.f;
    if (!((hw > th) || (he > th))) return 0.f;
    const float ze = S.z[e], zw = S.z[w];
    const float hhe = he + ze, hhw = hw + zw;
    const float hhep = he - th, hhwp = hw - th;
    if (hhe < zw) return hw > th ? 0.5440f * hw * fsqrt(gg * hw) : 0.f;
    if (hhw < ze) return he > th ? -0.544f * he * fsqrt(gg * he) : 0.f;
    if (hhep * hhwp < 0.f) {
        if ((he > 0.f) || (hw > 0.f)) {
            const float sg = copysignf(1.f, hhep - hhwp);
            const float hh3 = fmaxf(hhe, hhw) - fmaxf(ze, zw);
            return -sg * 0.350f * hh3 * fsqrt(2.f * gg * hh3);
        }
        return 0.f;
    }
    const float hm = 0.5f * (he + hw);
    const float u13 = gg * hm * sl.dt2dx * ((he - hw) + (ze - zw));
    const float* U = S.u;
    const int ui = (lr - 2) * U_W + (lc - 2);
    const float uc = U[ui], uS = U[ui + U_W], uN = U[ui - U_W];
    const float u11uur = 0.5f * (uS + uc), u11uul = 0.5f * (uc + uN);
    const float um0 = S.qx[e], umS = S.qx[e + LW], umN = S.qx[w];
    const float umr = u11uur * (umS + um0) * 0.5f + fabsf(u11uur) * (um0 - umS) * 0.5f;
    const float uml = u11uul * (um0 + umN) * 0.5f + fabsf(u11uul) * (umN - um0) * 0.5f;
    const float u11 = sl.dt2dx * (umr - uml);
    const float* V = S.v;
    const int vi = (lr - 2) * V_W + (lc - 2);
    const float v_e = V[vi], v_e1 = V[vi + 1], v_w = V[vi - V_W], v_w1 = V[vi - V_W + 1];
    float u12 = 0.f;
    if (c != 0) {
        const float u12vvu = 0.5f * (v_e1 + v_w1), u12vvd = 0.5f * (v_e + v_w);
        const float umE = S.qx[e + 1], umW = S.qx[e - 1];
        const float umu = u12vvu * (umE + um0) * 0.5f + fabsf(u12vvu) * (um0 - umE) * 0.5f;
        const float umd = u12vvd * (umW + um0) * 0.5f + fabsf(u12vvd) * (umW - um0) * 0.5f;
        u12 = sl.dt2dy * (umu - umd);
    }
    const float vva = 0.25f * (v_e + v_e1 + v_w + v_w1);
    const float sqx = fsqrt(uc * uc + vva * vva);
    float ram = 0.f;
    if (hm > th) {
        const float nf = 0.5f * (S.ntab[ie >> 1] + S.ntab[iw >> 1]);
        ram = gg * nf * nf * sqx * rpow_manning_f32(hm);
    }
    const float a = sl.dt2 * ram * 0.5f;
    return fdiv((1.f - a) * um0 + (-u11 - u12 - u13), 1.f + a);
}

/* y face between staged cells (lr, lc-1) "s" and (lr, lc) "n" */
__device__ __forceinline__ float flux_y32(const Smem32& S, const Scn32& P, const Slot32& sl, int lr, int lc,
                                          int r) {
    const int n = lr * LW + lc, so = n - 1;
    const float th = P.th, gg = P.g;
    const uint8_t in = S.info[lr * LWB + lc], is = S.info[lr * LWB + lc - 1];
    if (!(in & is & SW2D_I_ACTIVE)) return 0.f;
    const float hn = S.h[n], hs = S.h[so];
    if (!((hs > th) || (hn > th))) return 0.f;
    const float zn = S.z[n], zs = S.z[so];
    const float hhn = hn + zn, hhs = hs + zs;
    const float hhnp = hn - th, hhsp = hs - th;
    if (hhn < zs) return hs > th ? 0.5440f * hs * fsqrt(gg * hs) : 0.f;
    if (hhs < zn) return hn > th ? -0.544f * hn * fsqrt(gg * hn) : 0.f;
    if (hhnp * hhsp < 0.f) {
        if ((hn > 0.f) || (hs > 0.f)) {
            const float sg = copysignf(1.f, hhnp - hhsp);
            const float hh3 = fmaxf(hhn, hhs) - fmaxf(zn, zs);
            return -sg * 0.350f * hh3 * fsqrt(2.f * gg * hh3);
        }
        return 0.f;
    }
    const float hnf = 0.5f * (hn + hs);
    const float v13 = gg * hnf * sl.dt2dy * ((hn - hs) + (zn - zs));
    const float vn0 = S.qy[n];
    const float* U = S.u;
    const int ui = (lr - 2) * U_W + (lc - 2);
    const float ua = U[ui], ub = U[ui + U_W], uc = U[ui - 1], ud = U[ui + U_W - 1];
    float v11 = 0.f;
    if (r != 0) {
        const float v11uur = 0.5f * (ub + ud), v11uul = 0.5f * (ua + uc);
        const float vS = S.qy[n + LW], vN = S.qy[n - LW];
        const float vnr = v11uur * (vS + vn0) * 0.5f + fabsf(v11uur) * (vn0 - vS) * 0.5f;
        const float vnl = v11uul * (vn0 + vN) * 0.5f + fabsf(v11uul) * (vN - vn0) * 0.5f;
        v11 = sl.dt2dx * (vnr - vnl);
    }
    const float* V = S.v;
    const int vi = (lr - 2) * V_W + (lc - 2);
    const float vc = V[vi];
    const float v12vvu = 0.5f * (V[vi + 1] + vc), v12vvd = 0.5f * (vc + V[vi - 1]);
    const float vE = S.qy[n + 1], vW = S.qy[n - 1];
    const float vnu = v12vvu * (vE + vn0) * 0.5f + fabsf(v12vvu) * (vn0 - vE) * 0.5f;
    const float vnd = v12vvd * (vW + vn0) * 0.5f + fabsf(v12vvd) * (vW - vn0) * 0.5f;
    const float v12 = sl.dt2dy * (vnu - vnd);
    const float uua = 0.25f * (ua + ub + uc + ud);
    const float sqy = fsqrt(uua * uua + vc * vc);
    float ram = 0.f;
    if (hnf > th) {
        const float nf = 0.5f * (S.ntab[in >> 1] + S.ntab[is >> 1]);
        ram = gg * nf * nf * sqy * rpow_manning_f32(hnf);
    }
    const float a = sl.dt2 * ram * 0.5f;
    return fdiv((1.f - a) * vn0 + (-v11 - v12 - v13), 1.f + a);
}

__device__ __forceinline__ float pct_of(const Scn32& P, float ho) {
    return ho > P.ev_wl_min ? P.pct_lake : P.pct_land;
}

/* ---------------- the fused step ---------------------------------------- */

__global__ void __launch_bounds__(NT, 3) k32_step(const Scn32* __restrict__ scns, const int4* __restrict__ work,
                                                  Part32* __restrict__ part) {
    extern __shared__ unsigned char smem_raw[];
    Smem32& S = *reinterpret_cast<Smem32*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    const int tid = threadIdx.x;
    const int4 w = work[blockIdx.x];
    const Scn32& P = scns[w.x];
    Clock32* clk = P.clk;
    const Slot32 sl = clk->slot;
    if (!sl.active) {
        if (tid == 0) {
            Part32 z = {};
            part[blockIdx.x] = z;
        }
        return;
    }
    const int cur = sl.cur, nxt = cur ^ 1;
    const int tx = w.y, ty = w.z;
    const int c0 = tx * TC, r0 = ty * TR;

    /* self-check of the staging layout: a misaligned TMA destination would
     * fault, so record it and skip the tile instead */
    if (((smem_addr(S.h) | smem_addr(S.z) | smem_addr(S.qx) | smem_addr(S.qy) | smem_addr(S.info)) & 127u) != 0u) {
        if (tid == 0) atomicOr(&clk->status, 4);
        return;
    }
    if (tid == 0) {
        mbar_init(&S.bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) {
        const unsigned bytes = 4u * LH * LW * sizeof(float) + LH * LWB;
        mbar_arrive_expect_tx(&S.bar, bytes);
        /* staged origin (r0 - 4, c0 - 4) is padded coordinate (c0, r0) */
        tma_load_2d(S.h, &P.tm_h[cur], c0, r0, &S.bar);
        tma_load_2d(S.z, &P.tm_z, c0, r0, &S.bar);
        tma_load_2d(S.qx, &P.tm_qx[cur], c0, r0, &S.bar);
        tma_load_2d(S.qy, &P.tm_qy[cur], c0, r0, &S.bar);
        tma_load_2d(S.info, &P.tm_info, c0, r0, &S.bar);
    }
    if (tid < T32_MAXCLASS) S.ntab[tid] = P.ntab[tid];
    if (tid < 9) {
        const int dy = tid / 3 - 1, dx = tid % 3 - 1;
        const int ny = ty + dy, nx = tx + dx;
        float d = 0.f;
        if (ny >= 0 && ny < P.tiles_y && nx >= 0 && nx < P.tiles_x)
            d = P.datum[ny * P.tiles_x + nx] - P.datum[ty * P.tiles_x + tx];
        S.dd[tid] = d;
    }
    if (!wait_tile(&S.bar, clk)) return;
    __syncthreads();

    /* bed offsets of halo cells from the neighbouring tiles' datum to ours */
    for (int k = tid; k < LH * LW; k += NT) {
        const int lr = k / LW, lc = k - lr * LW;
        const int dy = lr < T32_H ? 0 : (lr >= T32_H + TR ? 2 : 1);
        const int dx = lc < T32_H ? 0 : (lc >= T32_H + TC ? 2 : 1);
        if (dy != 1 || dx != 1) S.z[k] += S.dd[dy * 3 + dx];
    }

    /* 1. face velocities, and the CFL face speeds of the tile's own faces
     *    (north and west faces of its cells between two active cells) */
    const float th = P.th;
    float sx = 0.f, sy = 0.f;
    for (int k = tid; k < U_H * U_W; k += NT) {
        const int lr = 2 + k / U_W, lc = 2 + k % U_W;
        const int r = r0 - T32_H + lr;
        const int i = lr * LW + lc;
        const float hm = (r == P.R) ? S.h[i - LW] : 0.5f * (S.h[i] + S.h[i - LW]);
        const float q = S.qx[i];
        const float u = (hm >= th && q != 0.f) ? fdiv(q, hm) : 0.f;
        S.u[k] = u;
        if (lr >= T32_H && lr < T32_H + TR && lc >= T32_H && lc < T32_H + TC && hm >= th &&
            (S.info[lr * LWB + lc] & S.info[(lr - 1) * LWB + lc] & SW2D_I_ACTIVE))
            sx = fmaxf(sx, (fabsf(u) + fsqrt(P.g * hm)) * P.rdx);
    }
    for (int k = tid; k < V_H * V_W; k += NT) {
        const int lr = 2 + k / V_W, lc = 2 + k % V_W;
        const int i = lr * LW + lc;
        const float hn = 0.5f * (S.h[i] + S.h[i - 1]);
        const float q = S.qy[i];
        const float v = (hn >= th && q != 0.f) ? fdiv(q, hn) : 0.f;
        S.v[k] = v;
        if (lr >= T32_H && lr < T32_H + TR && lc >= T32_H && lc < T32_H + TC && hn >= th &&
            (S.info[lr * LWB + lc] & S.info[lr * LWB + lc - 1] & SW2D_I_ACTIVE))
            sy = fmaxf(sy, (fabsf(v) + fsqrt(P.g * hn)) * P.rdy);
    }
    __syncthreads();

    /* 2a. x faces (need qx as the old discharge, so results wait in registers) */
    constexpr int NFX = (FX_H * FX_W + NT - 1) / NT;
    float fx[NFX];
#pragma unroll
    for (int j = 0; j < NFX; j++) {
        const int k = tid + j * NT;
        fx[j] = 0.f;
        if (k < FX_H * FX_W) {
            const int lr = 3 + k / FX_W, lc = 3 + k % FX_W;
            fx[j] = flux_x32(S, P, sl, lr, lc, r0 - T32_H + lr, c0 - T32_H + lc);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NFX; j++) {
        const int k = tid + j * NT;
        if (k < FX_H * FX_W) {
            const int lr = 3 + k / FX_W, lc = 3 + k % FX_W;
            S.qx[lr * LW + lc] = fx[j];
        }
    }
    /* 2b. y faces */
    constexpr int NFY = (FY_H * FY_W + NT - 1) / NT;
    float fy[NFY];
#pragma unroll
    for (int j = 0; j < NFY; j++) {
        const int k = tid + j * NT;
        fy[j] = 0.f;
        if (k < FY_H * FY_W) {
            const int lr = 3 + k / FY_W, lc = 3 + k % FY_W;
            fy[j] = flux_y32(S, P, sl, lr, lc, r0 - T32_H + lr);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < NFY; j++) {
        const int k = tid + j * NT;
        if (k < FY_H * FY_W) {
            const int lr = 3 + k / FY_W, lc = 3 + k % FY_W;
            S.qy[lr * LW + lc] = fy[j];
        }
    }
    __syncthreads();

    /* 3. provisional depth at t on the tile and its ring */
    const float rdx = P.rdx, rdy = P.rdy;
    for (int k = tid; k < D_H * D_W; k += NT) {
        const int lr = 3 + k / D_W, lc = 3 + k % D_W;
        const int i = lr * LW + lc;
        const uint8_t inf = S.info[lr * LWB + lc];
        uint8_t dry = 0;
        if (inf & SW2D_I_ACTIVE) {
            const float ho = S.h[i];
            float rr = sl.rr1;
            if (P.rainw) rr *= P.rainw[(size_t)(r0 + lr) * P.P + (c0 + lc)];
            const float ev = ho > P.ev_wl_min ? sl.ev1 : 0.f;
            const float hs = ho - sl.dt2 * ((S.qx[i + LW] - S.qx[i]) * rdx + (S.qy[i + 1] - S.qy[i]) * rdy -
                                            rr * pct_of(P, ho) + ev);
            dry = hs < th;
        }
        S.dry[k] = dry;
    }
    __syncthreads();

    /* 4. close outward faces of dry cells, final depth, write back */
    float clamp = 0.f, qout = 0.f, rain = 0.f, evc = 0.f;
    const int lc = T32_H + (tid % TC);
    const int c = c0 + (tid % TC);
#pragma unroll 2
    for (int j = 0; j < TR * TC / NT; j++) {
        const int lr = T32_H + tid / TC + j * (NT / TC);
        const int r = r0 + (lr - T32_H);
        if (r >= P.R || c >= P.C) continue;
        const int i = lr * LW + lc;
        const int di = (lr - 3) * D_W + (lc - 3);
        const uint8_t dc = S.dry[di];
        float fN = S.qx[i], fS = S.qx[i + LW], fW = S.qy[i], fE = S.qy[i + 1];
        if ((fN > 0.f && S.dry[di - D_W]) || (fN < 0.f && dc)) fN = 0.f;
        if ((fS > 0.f && dc) || (fS < 0.f && S.dry[di + D_W])) fS = 0.f;
        if ((fW > 0.f && S.dry[di - 1]) || (fW < 0.f && dc)) fW = 0.f;
        if ((fE > 0.f && dc) || (fE < 0.f && S.dry[di + 1])) fE = 0.f;
        const size_t g = (size_t)(r + T32_H) * P.P + (c + T32_H);
        const uint8_t inf = S.info[lr * LWB + lc];
        float hn = 0.f, kc = 0.f;
        if (inf & SW2D_I_ACTIVE) {
            const float ho = S.h[i];
            float wgt = P.rainw ? P.rainw[g] : 1.f;
            const float pct = pct_of(P, ho);
            const float ev = ho > P.ev_wl_min ? sl.ev2 : 0.f;
            const float dh = -sl.dt2 * ((fS - fN) * rdx + (fE - fW) * rdy - sl.rr2 * wgt * pct + ev);
            /* Kahan: the increment is small against the depth */
            const float y = dh - P.kc[g];
            const float t = ho + y;
            kc = (t - ho) - y;
            hn = t;
            if (hn < 0.f) {
                clamp -= hn;
                hn = 0.f;
                kc = 0.f;
            }
            if (P.ledger_cells) {
                rain += wgt * pct;
                evc += ho > P.ev_wl_min ? 1.f : 0.f;
            }
        }
        P.h[nxt][g] = hn;
        P.kc[g] = kc;
        P.qx[nxt][g] = fN;
        P.qy[nxt][g] = fW;
        if (r == P.R - 1) {
            P.qx[nxt][g + P.P] = fS;
            qout += fS;
        }
    }

    /* block reductions: warp sums in binary32, across warps in binary64 */
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sx = fmaxf(sx, __shfl_xor_sync(0xffffffffu, sx, o));
        sy = fmaxf(sy, __shfl_xor_sync(0xffffffffu, sy, o));
        clamp += __shfl_xor_sync(0xffffffffu, clamp, o);
        qout += __shfl_xor_sync(0xffffffffu, qout, o);
        rain += __shfl_xor_sync(0xffffffffu, rain, o);
        evc += __shfl_xor_sync(0xffffffffu, evc, o);
    }
    const int warp = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        S.red[warp][0] = clamp;
        S.red[warp][1] = qout;
        S.red[warp][2] = rain;
        S.red[warp][3] = evc;
        S.redf[warp][0] = sx;
        S.redf[warp][1] = sy;
    }
    __syncthreads();
    if (tid == 0) {
        Part32 pr = {};
        float mx = 0.f, my = 0.f;
        for (int k = 0; k < NT / 32; k++) {
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
        const size_t g = (size_t)(r + T32_H) * P.P + (c + T32_H);
        if (!(P.info[g] & SW2D_I_ACTIVE)) continue;
        const float hh = P.h[cur][g];
        vol += (double)hh - (double)P.kc[g];
        if (r > 0 && (P.info[g - P.P] & SW2D_I_ACTIVE)) {
            const float hm = 0.5f * (hh + P.h[cur][g - P.P]);
            const float q = P.qx[cur][g];
            if (hm >= th) sx = fmaxf(sx, (fabsf(q != 0.f ? q / hm : 0.f) + fsqrt(P.g * hm)) * P.rdx);
        }
        if (c > 0 && (P.info[g - 1] & SW2D_I_ACTIVE)) {
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
    cudaError_t e = cudaFuncSetAttribute(k32_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fp32_smem_bytes());
    return e == cudaSuccess ? 0 : -1;
}

void fp32_launch_iteration(const Scn32* d_scn, int nscn, const int4* d_work, int nwork, Part32* d_part,
                           cudaStream_t s) {
    if (nwork > 0) k32_step<<<nwork, NT, fp32_smem_bytes(), s>>>(d_scn, d_work, d_part);
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
