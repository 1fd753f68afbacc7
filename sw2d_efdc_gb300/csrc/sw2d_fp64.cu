/* FP64 SW2D step on sm_103a: the plain path whose results match the
 * reference's own kernels (SW2D-EFDC.cu:97-725).
 *
 * GB300's FP64 pipe runs at ~1/64 of the FP32 rate, so this path is bound by
 * FP64 instructions, not HBM.  The step is therefore split so that nothing
 * FP64 is computed twice:
 *   k64_flux   : new x/y face discharges of every face (flux, :97-353) from the
 *                stored face velocities uu1/vv1 of the previous iteration
 *   k64_hstar  : provisional depth (continuity at t, :602-664) -> one byte
 *                per cell "active and h* < th" (the treat_error predicate)
 *   k64_depth  : closes outward faces of those cells on the fly (treat_error,
 *                :695-725, restated per face), final depth at t+dt, FP64
 *                volume / rain / clamp / outlet sums and the CFL speed
 *                maximum by block reduction; the last block reduces the
 *                per-block partials in a fixed order and prepares the next
 *                iteration's length and forcing on the device
 *   k64_facevel: writes the closed faces back and the face velocities
 *                uu1 = qx/hm, vv1 = qy/hn of the new state (hm_hn, uu1_vv1,
 *                :362-452); forward (:670-693) is a buffer swap.
 * Compiled with --fmad=false: every expression is evaluated with the same
 * roundings as the CPU oracle (gcc -ffp-contract=off), explicit fma() only
 * where sw2d_math.h spells it.
 */
#include "sw2d_internal.h"
#include "sw2d_math.h"

namespace sw2d {

#define H SW2D_HALO

__device__ __forceinline__ double series_at(const double* v, int n, double dts, double time, int mode) {
    double r;
    int it;
    if (mode == 0) { /* SW2D-EFDC.cu:546-551 */
        if (time <= 1.00) {
            r = v[0] * time;
        } else {
            it = (int)(time / dts);
            if (it + 1 > n) it = n;
            r = v[it] + (v[it + 1] - v[it]) / (dts * (time - dts * (it)));
        }
    } else if (mode == 1) {
        it = (int)(time / dts);
        if (it + 1 > n) it = n;
        r = v[it] + (v[it + 1] - v[it]) * ((time - dts * (it)) / dts);
    } else {
        it = (int)(time / dts);
        if (it > n) it = n;
        r = v[it];
    }
    return r;
}

__device__ __forceinline__ double source_at(const StepParams& p, int i, double time) {
    double q;
    const double* Q = p.srcq;
    const int ns = p.nsrc;
    if (p.series_mode == 0) { /* stream_flow SW2D-EFDC.cu:531-538 */
        if (time <= 1.00) {
            q = Q[i] * time;
        } else {
            int it = (int)(time / p.dtoq);
            if (it + 1 > p.nq) it = p.nq;
            q = Q[(size_t)it * ns + i] + (Q[(size_t)(it + 1) * ns + i] - Q[(size_t)it * ns + i]) /
                                             (p.dtoq * (time - p.dtoq * (it)));
        }
    } else {
        int it = (int)(time / p.dtoq);
        if (it + 1 > p.nq) it = p.nq;
        double a = Q[(size_t)it * ns + i];
        if (p.series_mode == 1) {
            double b = Q[(size_t)(it + 1) * ns + i];
            q = a + (b - a) * ((time - p.dtoq * (it)) / p.dtoq);
        } else {
            q = a;
        }
    }
    return q / (p.dx * p.dy);
}

/* Length and forcing of the iteration that starts at time t (run by one
 * thread).  FIXED: the reference's loop (:4798, :4838, :4876).  CFL:
 * min(dt_max, cfl/s), shortened to end exactly at t_end. */
__device__ void prepare_slot(const StepParams& p, Slot* s, double t, double smax, double t_end) {
    double dt2, tm, tn;
    int active;
    if (p.dt_mode == 0) {
        double dt = p.dt_fixed;
        active = (t + dt <= t_end);
        dt2 = 2.00 * dt;
        tm = t + dt;
        tn = tm + dt;
    } else {
        active = (t < t_end);
        dt2 = smax > 0 ? fmin(p.dt_max, p.cfl / smax) : p.dt_max;
        if (t + dt2 > t_end) dt2 = t_end - t;
        tm = t + 0.5 * dt2;
        tn = t + dt2;
    }
    s->t = t;
    s->t_mid = tm;
    s->t_next = tn;
    s->dt2 = dt2;
    s->dt2dx = dt2 / p.dx;
    s->dt2dy = dt2 / p.dy;
    s->active = active;
    s->rr1 = series_at(p.rain, p.nrain, p.dtrain, t, p.series_mode) / (p.dtrain * 1000.0);
    s->rr2 = series_at(p.rain, p.nrain, p.dtrain, tm, p.series_mode) / (p.dtrain * 1000.0);
    if (p.evap) {
        s->ev1 = series_at(p.evap, p.nevap, p.dtrain, t, p.series_mode) / (p.dtrain * 1000.0);
        s->ev2 = series_at(p.evap, p.nevap, p.dtrain, tm, p.series_mode) / (p.dtrain * 1000.0);
    } else {
        s->ev1 = s->ev2 = 0.0;
    }
    for (int k = 0; k < p.nsrc; k++) {
        s->ql1[k] = source_at(p, k, t);
        s->ql2[k] = source_at(p, k, tm);
    }
}

/* ------------------------------------------------------------------------ */
/* flux: SW2D-EFDC.cu:97-353                                                 */

__device__ __forceinline__ double face_manning(const StepParams& p, size_t a, size_t b) {
    if (!p.mcls) return p.manning;
    return 0.50 * (p.mtab[p.mcls[a]] + p.mtab[p.mcls[b]]);
}

__device__ __forceinline__ double friction(const StepParams& p, double nf, double sq, double hm) {
    /* :193-198; the division by pow(hm, 1.333333) as a product with hm^-1.333333 */
    if (hm <= p.th) return 0.00;
    return (p.g * nf * nf * sq) * sw2d_rpow_manning(hm);
}

/* x face between cell w = (r-1, c) and e = (r, c), positive southward */
__device__ __forceinline__ double flux_x(const StepParams& p, const double* __restrict__ h,
                                         const double* __restrict__ umo, int r, int c, size_t e,
                                         double dt2, double dt2dx, double dt2dy) {
    const double th = p.th, gg = p.g;
    const int P = p.P;
    const size_t w = e - P;
    const double* __restrict__ z = p.z;
    const double* __restrict__ uu1 = p.uu1;
    const double* __restrict__ vv1 = p.vv1;
    const uint8_t fe = p.flags[e], fw = p.flags[w];
    const double he = h[e], hw = h[w];
    if (r == p.R && p.outflow_south) {
        if ((fw & SW2D_F_ACTIVE) && hw > th) return 0.5440 * hw * sqrt(gg * hw);
        return 0;
    }
    if (!(fe & SW2D_F_ACTIVE) || !(fw & SW2D_F_ACTIVE)) return 0;
    if (!((hw > th) || (he > th))) return 0;
    const double ze = z[e], zw = z[w];
    const double hhe = he + ze;
    const double hhw = hw + zw;
    const double hhep = he - th;
    const double hhwp = hw - th;
    if (hhe < zw) {
        if (hw > th) return 0.5440 * hw * sqrt(gg * hw);
        return 0;
    } else if (hhw < ze) {
        if (he > th) return -0.544 * he * sqrt(gg * he);
        return 0;
    } else if (hhep * hhwp < 0) {
        if ((he > 0) || (hw > 0)) {
            double hhan = hhep - hhwp;
            double sgnm = copysign(1.0, hhan);
            double hh3 = fmax(hhe, hhw) - fmax(ze, zw);
            return -sgnm * 0.350 * hh3 * sqrt(2.00 * gg * hh3);
        }
        return 0;
    }
    const double hm = 0.50 * (he + hw);
    const double u13 = gg * hm * dt2dx * (hhe - hw - zw);
    const double uc = uu1[e];
    const double u11uur = 0.50 * (uu1[e + P] + uc);
    const double u11uul = 0.50 * (uc + uu1[w]);
    const double um0 = umo[e], umS = umo[e + P], umN = umo[w];
    const double umr = u11uur * (umS + um0) * 0.50 + fabs(u11uur) * (um0 - umS) * 0.50;
    const double uml = u11uul * (um0 + umN) * 0.50 + fabs(u11uul) * (umN - um0) * 0.50;
    const double u11 = dt2dx * (umr - uml);
    const double v_e = vv1[e], v_e1 = vv1[e + 1], v_w = vv1[w], v_w1 = vv1[w + 1];
    double u12;
    if (c == 0) {
        u12 = 0;
    } else {
        const double u12vvu = 0.50 * (v_e1 + v_w1);
        const double u12vvd = 0.50 * (v_e + v_w);
        const double umE = umo[e + 1], umW = umo[e - 1];
        const double umu = u12vvu * (umE + um0) * 0.50 + fabs(u12vvu) * (um0 - umE) * 0.50;
        const double umd = u12vvd * (umW + um0) * 0.50 + fabs(u12vvd) * (umW - um0) * 0.50;
        u12 = dt2dy * (umu - umd);
    }
    const double vva = 0.250 * (v_e + v_e1 + v_w + v_w1);
    const double sqx = sqrt(uc * uc + vva * vva);
    const double ram = friction(p, face_manning(p, e, w), sqx, hm);
    return ((1.00 - dt2 * ram * 0.50) * um0 + (-u11 - u12 - u13)) / (1.00 + dt2 * ram * 0.50);
}

/* y face between cell s = (r, c-1) and n = (r, c), positive eastward */
__device__ __forceinline__ double flux_y(const StepParams& p, const double* __restrict__ h,
                                         const double* __restrict__ vno, int r, int c, size_t n,
                                         double dt2, double dt2dx, double dt2dy) {
    const double th = p.th, gg = p.g;
    const int P = p.P;
    const size_t so = n - 1;
    const double* __restrict__ z = p.z;
    const double* __restrict__ uu1 = p.uu1;
    const double* __restrict__ vv1 = p.vv1;
    const uint8_t fn = p.flags[n], fs = p.flags[so];
    if (!(fn & SW2D_F_ACTIVE) || !(fs & SW2D_F_ACTIVE)) return 0;
    const double hn = h[n], hs = h[so];
    if (!((hs > th) || (hn > th))) return 0;
    const double zn = z[n], zs = z[so];
    const double hhn = hn + zn;
    const double hhs = hs + zs;
    const double hhnp = hn - th;
    const double hhsp = hs - th;
    if (hhn < zs) {
        if (hs > th) return 0.5440 * hs * sqrt(gg * hs);
        return 0;
    } else if (hhs < zn) {
        if (hn > th) return -0.544 * hn * sqrt(gg * hn);
        return 0;
    } else if (hhnp * hhsp < 0) {
        if ((hn > 0) || (hs > 0)) {
            double hhan = hhnp - hhsp;
            double sgnm = copysign(1.0, hhan);
            double hh3 = fmax(hhn, hhs) - fmax(zn, zs);
            return -sgnm * 0.350 * hh3 * sqrt(2.00 * gg * hh3);
        }
        return 0;
    }
    const double hnf = 0.50 * (hn + hs);
    const double v13 = gg * hnf * dt2dy * (hhn - hs - zs);
    const double vn0 = vno[n];
    const double ua = uu1[n], ub = uu1[n + P], uc = uu1[n - 1], ud = uu1[n + P - 1];
    double v11;
    if (r == 0) {
        v11 = 0;
    } else {
        const double v11uur = 0.50 * (ub + ud);
        const double v11uul = 0.50 * (ua + uc);
        const double vS = vno[n + P], vN = vno[n - P];
        const double vnr = v11uur * (vS + vn0) * 0.50 + fabs(v11uur) * (vn0 - vS) * 0.50;
        const double vnl = v11uul * (vn0 + vN) * 0.50 + fabs(v11uul) * (vN - vn0) * 0.50;
        v11 = dt2dx * (vnr - vnl);
    }
    const double vc = vv1[n];
    const double v12vvu = 0.50 * (vv1[n + 1] + vc);
    const double v12vvd = 0.50 * (vc + vv1[n - 1]);
    const double vE = vno[n + 1], vW = vno[n - 1];
    const double vnu = v12vvu * (vE + vn0) * 0.50 + fabs(v12vvu) * (vn0 - vE) * 0.50;
    const double vnd = v12vvd * (vW + vn0) * 0.50 + fabs(v12vvd) * (vW - vn0) * 0.50;
    const double v12 = dt2dy * (vnu - vnd);
    const double uua = 0.250 * (ua + ub + uc + ud);
    const double sqy = sqrt(uua * uua + vc * vc);
    const double ram = friction(p, face_manning(p, n, so), sqy, hnf);
    return ((1.00 - dt2 * ram * 0.50) * vn0 + (-v11 - v12 - v13)) / (1.00 + dt2 * ram * 0.50);
}

__device__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* sm);
__device__ float block_max_f32_all(float v, float* sm);

/* CFL speed contribution of one face of the entering state: (|velocity| +
 * sqrt(g * mean depth)) / spacing for faces between two active cells whose
 * mean depth is >= th (the oracle's cfl_speed, same operations). */
__device__ __forceinline__ double face_speed(double vel, double hm, double g, double rd) {
    return (fabs(vel) + sqrt(g * hm)) * rd;
}

/* exact block maximum of face speeds: binary32 estimate for every face,
 * binary64 only for the faces within 1e-5 of the block's binary32 maximum */
__device__ __forceinline__ unsigned long long block_face_speed_max(bool ok, double vel, double hm, double g,
                                                                   double rd, float* smf,
                                                                   unsigned long long* smu) {
    const float s32 = ok ? (fabsf((float)vel) + sqrtf((float)g * (float)hm)) * (float)rd : 0.0f;
    const float m32 = block_max_f32_all(s32, smf);
    unsigned long long bits = 0ull;
    if (ok && s32 >= m32 * 0.99999f) bits = (unsigned long long)__double_as_longlong(face_speed(vel, hm, g, rd));
    return block_max_u64(bits, smu);
}

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_flux(StepParams p, int cur) {
    __shared__ float smf[SW2D_BX * SW2D_BY / 32];
    __shared__ unsigned long long smu[SW2D_BX * SW2D_BY / 32];
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    const int nxt = cur ^ 1;
    const Slot& s = p.clk->slot[cur];
    bool okx = false, oky = false;
    double hmx = 0, hmy = 0, vx = 0, vy = 0;
    if (r <= p.R && c <= p.C) {
        const size_t i = (size_t)(r + H) * p.P + (c + H);
        if (!s.active) {
            if (c < p.C) p.qx[nxt][i] = p.qx[cur][i];
            if (r < p.R) p.qy[nxt][i] = p.qy[cur][i];
        } else {
            const double dt2 = s.dt2, dt2dx = s.dt2dx, dt2dy = s.dt2dy;
            const double* __restrict__ h = p.h[cur];
            if (c < p.C) p.qx[nxt][i] = flux_x(p, h, p.qx[cur], r, c, i, dt2, dt2dx, dt2dy);
            if (r < p.R) p.qy[nxt][i] = flux_y(p, h, p.qy[cur], r, c, i, dt2, dt2dx, dt2dy);
            if (p.dt_mode == 1) {
                const uint8_t fc = p.flags[i];
                if (c < p.C && r > 0 && r < p.R && (fc & p.flags[i - p.P] & SW2D_F_ACTIVE)) {
                    hmx = 0.50 * (h[i] + h[i - p.P]);
                    okx = hmx >= p.th;
                    vx = p.uu1[i];
                }
                if (r < p.R && c > 0 && c < p.C && (fc & p.flags[i - 1] & SW2D_F_ACTIVE)) {
                    hmy = 0.50 * (h[i] + h[i - 1]);
                    oky = hmy >= p.th;
                    vy = p.vv1[i];
                }
            }
        }
    }
    if (p.dt_mode == 1) {
        const unsigned long long sx = block_face_speed_max(okx, vx, hmx, p.g, p.rdx, smf, smu);
        const unsigned long long sy = block_face_speed_max(oky, vy, hmy, p.g, p.rdy, smf, smu);
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            const int b = blockIdx.y * gridDim.x + blockIdx.x;
            p.partials_f[2 * b] = __longlong_as_double((long long)sx);
            p.partials_f[2 * b + 1] = __longlong_as_double((long long)sy);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* continuity: SW2D-EFDC.cu:602-664                                          */

__device__ __forceinline__ double continuity(const StepParams& p, size_t i, uint8_t f, double ho,
                                             double divx, double divy, double dt2, double rr,
                                             double ev, const double* ql, double* raw,
                                             double* rain_term) {
    double pct, evapo;
    if (ho > p.ev_wl_min) {
        pct = p.pct_lake;
        evapo = ev;
    } else {
        pct = p.pct_land;
        evapo = 0.000;
    }
    const double rcell = p.rainw ? rr * (double)p.rainw[i] : rr;
    double qli = 0.0;
    if (f & SW2D_F_SOURCE) {
        for (int k = 0; k < p.nsrc; k++)
            if (p.src_idx[k] == (int)i) qli = ql[k];
    }
    double hn = ho - dt2 * (sw2d_div_const(divx, p.dx, p.rdx) + sw2d_div_const(divy, p.dy, p.rdy) - qli -
                            rcell * pct + evapo);
    *raw = hn;
    *rain_term = rcell * pct;
    hn = fmax(hn, 0.00);
    if (!(f & SW2D_F_ACTIVE)) hn = 0.00;
    return hn;
}

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_hstar(StepParams p, int cur) {
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    if (r >= p.R || c >= p.C) return;
    const Slot& s = p.clk->slot[cur];
    if (!s.active) return;
    const int nxt = cur ^ 1;
    const size_t i = (size_t)(r + H) * p.P + (c + H);
    const uint8_t f = p.flags[i];
    const double* __restrict__ fx = p.qx[nxt];
    const double* __restrict__ fy = p.qy[nxt];
    double raw, rt;
    const double hs = continuity(p, i, f, p.h[cur][i], fx[i + p.P] - fx[i], fy[i + 1] - fy[i], s.dt2,
                                 s.rr1, s.ev1, s.ql1, &raw, &rt);
    p.drys[i] = (uint8_t)((f & SW2D_F_ACTIVE) && hs < p.th);
}

/* ------------------------------------------------------------------------ */
/* block reductions (fixed order: deterministic for a given grid)            */

#define NWARP (SW2D_BX * SW2D_BY / 32)

__device__ __forceinline__ int tid_linear() { return threadIdx.y * SW2D_BX + threadIdx.x; }

__device__ __forceinline__ double block_sum(double v, double* sm) {
    const int lane = tid_linear() & 31, warp = tid_linear() >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = lane < NWARP ? sm[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    }
    return t; /* valid in thread 0 */
}

__device__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* sm) {
    const int lane = tid_linear() & 31, warp = tid_linear() >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long u = __shfl_down_sync(0xffffffffu, v, o);
        v = u > v ? u : v;
    }
    __syncthreads();
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (warp == 0) {
        t = lane < NWARP ? sm[lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long u = __shfl_down_sync(0xffffffffu, t, o);
            t = u > t ? u : t;
        }
    }
    return t; /* valid in thread 0 */
}

__device__ float block_max_f32_all(float v, float* sm) {
    const int lane = tid_linear() & 31, warp = tid_linear() >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    float t = sm[0];
#pragma unroll
    for (int k = 1; k < NWARP; k++) t = fmaxf(t, sm[k]);
    return t; /* valid in every thread */
}

#define NPART 4 /* rain, evap, qout, s_max bits */

/* Final reduction over the per-block partials by the last block to finish,
 * then the iteration's ledger update and the next slot. */
__device__ void finish_iteration(const StepParams& p, int cur, int nblocks) {
    __shared__ bool last;
    __shared__ double smd[NWARP];
    __shared__ unsigned long long smu[NWARP];
    __threadfence();
    const int tid = tid_linear();
    if (tid == 0) {
        unsigned int ticket = atomicAdd(&p.clk->counter, 1u);
        last = (ticket == (unsigned)nblocks - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double vr = 0.0, ve = 0.0, vq = 0.0;
    unsigned long long vs = 0ull;
    for (int b = tid; b < nblocks; b += SW2D_BX * SW2D_BY) {
        const volatile double* pb = p.partials + (size_t)b * NPART;
        vr += pb[0];
        ve += pb[1];
        vq += pb[2];
    }
    if (p.ledger_cells) {
        vr = block_sum(vr, smd);
        ve = block_sum(ve, smd);
    }
    if (p.outflow_south) vq = block_sum(vq, smd);
    /* CFL speed of the state this iteration started from, from k64_flux */
    unsigned long long ux = 0ull, uy = 0ull;
    if (p.dt_mode == 1) {
        for (int b = tid; b < p.nblocks_faces; b += SW2D_BX * SW2D_BY) {
            const volatile double* pb = p.partials_f + (size_t)b * 2;
            unsigned long long a = (unsigned long long)__double_as_longlong(pb[0]);
            unsigned long long c = (unsigned long long)__double_as_longlong(pb[1]);
            ux = a > ux ? a : ux;
            uy = c > uy ? c : uy;
        }
        ux = block_max_u64(ux, smu);
        uy = block_max_u64(uy, smu);
    }
    (void)vs;
    if (tid == 0) {
        DevClock* clk = p.clk;
        const Slot& s = clk->slot[cur];
        if (s.active) {
            const double dt2 = s.dt2;
            const double smax = __longlong_as_double((long long)ux) + __longlong_as_double((long long)uy);
            double src = 0.0;
            for (int k = 0; k < p.nsrc; k++) src += s.ql2[k];
            const double rain = p.ledger_cells ? vr : s.rr2 * p.rain_static;
            clk->led[LED_RAIN] += dt2 * rain * p.area;
            clk->led[LED_EVAP] += dt2 * ve * p.area;
            clk->led[LED_SOURCE] += dt2 * src * p.area;
            clk->led[LED_QOUT] = vq * p.dy;
            clk->led[LED_OUTFLOW] += dt2 * clk->led[LED_QOUT];
            clk->led[LED_DTLAST] = dt2;
            clk->led[LED_SMAX] = smax;
            if (!isfinite(smax) || !isfinite(vq)) clk->status |= 1;
            clk->t = s.t_next;
            clk->s_max = smax;
            clk->iters += 1;
            if (p.outlet) {
                long long k = clk->outlet_n % p.outlet_cap;
                p.outlet[2 * k] = s.t_next;
                p.outlet[2 * k + 1] = clk->led[LED_QOUT];
                clk->outlet_n += 1;
            }
            prepare_slot(p, &clk->slot[cur ^ 1], clk->t, clk->s_max, clk->t_end);
        } else {
            clk->slot[cur ^ 1] = s;
        }
        clk->counter = 0;
    }
}

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_depth(StepParams p, int cur) {
    __shared__ double smd[NWARP];
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    const int nxt = cur ^ 1;
    const Slot& s = p.clk->slot[cur];
    double vr = 0.0, ve = 0.0, vq = 0.0;
    bool wet = false;
    double fN = 0, fS = 0, fW = 0, fE = 0, hn = 0;
    if (r < p.R && c < p.C) {
        const int P = p.P;
        const size_t i = (size_t)(r + H) * P + (c + H);
        if (!s.active) {
            p.h[nxt][i] = p.h[cur][i];
        } else {
            const uint8_t f = p.flags[i];
            const double* __restrict__ fx = p.qx[nxt];
            const double* __restrict__ fy = p.qy[nxt];
            const uint8_t* __restrict__ d = p.drys;
            const uint8_t dc = d[i];
            /* treat_error per face: a face carrying water out of a cell whose
             * provisional depth fell below th is closed (:704-719) */
            fN = fx[i];
            fS = fx[i + P];
            fW = fy[i];
            fE = fy[i + 1];
            if ((fN > 0 && d[i - P]) || (fN < 0 && dc)) fN = 0;
            if ((fS > 0 && dc) || (fS < 0 && d[i + P])) fS = 0;
            if ((fW > 0 && d[i - 1]) || (fW < 0 && dc)) fW = 0;
            if ((fE > 0 && dc) || (fE < 0 && d[i + 1])) fE = 0;
            const double ho = p.h[cur][i];
            double raw, rt;
            hn = continuity(p, i, f, ho, fS - fN, fE - fW, s.dt2, s.rr2, s.ev2, s.ql2, &raw, &rt);
            p.h[nxt][i] = hn;
            if (f & SW2D_F_ACTIVE) {
                if (raw < 0) atomicAdd(&p.clk->led[LED_CLAMP], -raw * p.area); /* max(h, 0) gain */
                if (p.ledger_cells) {
                    vr = rt;
                    ve = (ho > p.ev_wl_min) ? s.ev2 : 0.0;
                }
                if (r == p.R - 1) vq = fS;
                wet = hn >= p.th;
            }
        }
    }
    double pr = 0.0, pe = 0.0, pq = 0.0;
    if (p.ledger_cells) {
        pr = block_sum(vr, smd);
        pe = block_sum(ve, smd);
    }
    if (p.outflow_south && (blockIdx.y + 1) * SW2D_BY >= p.R) pq = block_sum(vq, smd);
    (void)wet;
    const int tid = tid_linear();
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
        double* pb = p.partials + (size_t)b * NPART;
        pb[0] = pr;
        pb[1] = pe;
        pb[2] = pq;
    }
    finish_iteration(p, cur, gridDim.x * gridDim.y);
}

/* Volume (sum of h over active cells) and, with full, the CFL speed of the
 * current state (face rule of k64_flux); the last block stores them and
 * prepares the next slot. */
__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_prime(StepParams p, int cur, int full) {
    __shared__ double smd[NWARP];
    __shared__ float smf[NWARP];
    __shared__ unsigned long long smu[NWARP];
    __shared__ bool last;
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    double vol = 0.0;
    bool okx = false, oky = false;
    double hmx = 0, hmy = 0, vx = 0, vy = 0;
    if (full && r < p.R && c < p.C) {
        const int P = p.P;
        const size_t i = (size_t)(r + H) * P + (c + H);
        const double* h = p.h[cur];
        const uint8_t fc = p.flags[i];
        if (fc & SW2D_F_ACTIVE) {
            vol = h[i];
            if (r > 0 && (p.flags[i - P] & SW2D_F_ACTIVE)) {
                hmx = 0.50 * (h[i] + h[i - P]);
                okx = hmx >= p.th;
                vx = p.uu1[i];
            }
            if (c > 0 && (p.flags[i - 1] & SW2D_F_ACTIVE)) {
                hmy = 0.50 * (h[i] + h[i - 1]);
                oky = hmy >= p.th;
                vy = p.vv1[i];
            }
        }
    }
    vol = block_sum(vol, smd);
    const unsigned long long sx = block_face_speed_max(okx, vx, hmx, p.g, p.rdx, smf, smu);
    const unsigned long long sy = block_face_speed_max(oky, vy, hmy, p.g, p.rdy, smf, smu);
    const int tid = tid_linear();
    const int b = blockIdx.y * gridDim.x + blockIdx.x;
    if (tid == 0) {
        p.partials[(size_t)b * NPART + 0] = vol;
        p.partials[(size_t)b * NPART + 1] = __longlong_as_double((long long)sx);
        p.partials[(size_t)b * NPART + 2] = __longlong_as_double((long long)sy);
    }
    __threadfence();
    if (tid == 0) last = (atomicAdd(&p.clk->counter, 1u) == gridDim.x * gridDim.y - 1);
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int nb = gridDim.x * gridDim.y;
    double v = 0.0;
    unsigned long long ux = 0ull, uy = 0ull;
    for (int bb = tid; bb < nb; bb += SW2D_BX * SW2D_BY) {
        const volatile double* pb = p.partials + (size_t)bb * NPART;
        v += pb[0];
        unsigned long long a = (unsigned long long)__double_as_longlong(pb[1]);
        unsigned long long w = (unsigned long long)__double_as_longlong(pb[2]);
        ux = a > ux ? a : ux;
        uy = w > uy ? w : uy;
    }
    v = block_sum(v, smd);
    ux = block_max_u64(ux, smu);
    uy = block_max_u64(uy, smu);
    if (tid == 0) {
        DevClock* clk = p.clk;
        /* full: 1 = volume only (the clock is left alone), 2 = initial state
         * (volume origin, CFL speed and the first slot), 0 = slot only */
        if (full) clk->led[LED_VOLUME] = v * p.area;
        if (full == 2) {
            clk->s_max = __longlong_as_double((long long)ux) + __longlong_as_double((long long)uy);
            clk->led[LED_SMAX] = clk->s_max;
            clk->led[LED_VOLUME0] = clk->led[LED_VOLUME];
        }
        if (full != 1) prepare_slot(p, &clk->slot[cur], clk->t, clk->s_max, clk->t_end);
        clk->counter = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* hm_hn + uu1_vv1: SW2D-EFDC.cu:362-452, with the closed faces written back  */

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_facevel(StepParams p, int cur, int clip) {
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    if (r > p.R || c > p.C) return;
    const int nxt = clip ? (cur ^ 1) : cur;
    if (clip && !p.clk->slot[cur].active) return;
    const int P = p.P;
    const size_t i = (size_t)(r + H) * P + (c + H);
    const double* __restrict__ h = p.h[nxt];
    const uint8_t* __restrict__ d = p.drys;
    const double th = p.th;
    if (c < p.C) {
        double F = p.qx[nxt][i];
        if (clip) {
            const double F0 = F;
            if ((F0 > 0 && d[i - P]) || (F0 < 0 && d[i])) F = 0;
            if (F != F0) p.qx[nxt][i] = F;
        }
        double hm;
        if (r == 0) hm = h[i];
        else if (r == p.R) hm = h[i - P];
        else hm = 0.50 * (h[i] + h[i - P]);
        p.uu1[i] = (hm >= th) ? (F == 0 ? F : F / hm) : 0.00; /* 0/hm is 0 of F's sign */
    }
    if (r < p.R) {
        double F = p.qy[nxt][i];
        if (clip) {
            const double F0 = F;
            if ((F0 > 0 && d[i - 1]) || (F0 < 0 && d[i])) F = 0;
            if (F != F0) p.qy[nxt][i] = F;
        }
        double hn;
        if (c == 0) hn = h[i];
        else if (c == p.C) hn = h[i - 1];
        else hn = 0.50 * (h[i] + h[i - 1]);
        p.vv1[i] = (hn >= th) ? (F == 0 ? F : F / hn) : 0.0;
    }
}

/* Reference-layout velocities for output: uu_vv (:458-483), uua_vva (:489-522). */
__global__ void k64_cellvel(StepParams p, int cur, double* uu, double* vv, double* uua, double* vva) {
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    if (r >= p.R || c >= p.C) return;
    const int P = p.P;
    const size_t i = (size_t)(r + H) * P + (c + H);
    const size_t k = (size_t)r * p.C + c;
    const double* u1 = p.uu1;
    const double* v1 = p.vv1;
    if (uu || vv) {
        double a = 0, b = 0;
        if (p.h[cur][i] >= p.th) {
            a = (u1[i + P] + u1[i]) / 2.00;
            b = (v1[i + 1] + v1[i]) / 2.00;
        }
        if (uu) uu[k] = a;
        if (vv) vv[k] = b;
    }
    if (uua) uua[k] = (c > 0) ? 0.250 * (u1[i] + u1[i + P] + u1[i - 1] + u1[i + P - 1]) : 0.50 * (u1[i] + u1[i + P]);
    if (vva) vva[k] = (r > 0) ? 0.250 * (v1[i] + v1[i + 1] + v1[i - P] + v1[i - P + 1]) : 0.50 * (v1[i] + v1[i + 1]);
}

/* Boundary-discharge sample (couple_BC_efdc, SW2D-EFDC.cu:728-1067): one
 * thread per boundary face.  North/south faces use uua and east/west faces
 * vva at the catchment cell, as the reference's call passes them
 * (SW2D-EFDC.cu:4909, signature :728); inflow to the lake only. */
__global__ void k_couple(StepParams p, int n, const int* __restrict__ faces, int lagged, int initial,
                         double* __restrict__ vel_prev, double* __restrict__ q) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int P = p.P;
    const int i = faces[2 * k], side = faces[2 * k + 1];
    const int r = i / P - H, c = i % P - H;
    const double* u1 = p.uu1;
    const double* v1 = p.vv1;
    double vnow;
    if (side <= 1)
        vnow = (c > 0) ? 0.250 * (u1[i] + u1[i + P] + u1[i - 1] + u1[i + P - 1]) : 0.50 * (u1[i] + u1[i + P]);
    else
        vnow = (r > 0) ? 0.250 * (v1[i] + v1[i + 1] + v1[i - P] + v1[i - P + 1]) : 0.50 * (v1[i] + v1[i + 1]);
    const double v = initial ? 0.0 : (lagged ? vel_prev[k] : vnow);
    const double hh = p.h[0][i];
    double out;
    switch (side) {
    case 1: out = (v < 0) ? -v * hh * p.dx : 0.00; break; /* south :760-767 */
    case 0: out = (v > 0) ? v * hh * p.dx : 0.00; break;  /* north :777-784 */
    case 2: out = (v < 0) ? -v * hh * p.dy : 0.00; break; /* east :794-801 */
    default: out = (v > 0) ? v * hh * p.dy : 0.00; break; /* west :812-819 */
    }
    q[k] = out;
    vel_prev[k] = vnow;
}

void launch_couple(const StepParams& p, int nfaces, const int* faces, int lagged, int initial, double* vel_prev,
                   double* q, cudaStream_t s) {
    k_couple<<<(nfaces + 127) / 128, 128, 0, s>>>(p, nfaces, faces, lagged, initial, vel_prev, q);
}

/* ------------------------------------------------------------------------ */

static dim3 grid_faces(const StepParams& p) {
    return dim3((p.C + 1 + SW2D_BX - 1) / SW2D_BX, (p.R + 1 + SW2D_BY - 1) / SW2D_BY);
}
static dim3 grid_cells(const StepParams& p) {
    return dim3((p.C + SW2D_BX - 1) / SW2D_BX, (p.R + SW2D_BY - 1) / SW2D_BY);
}

int fp64_kernels_per_iteration() { return 4; }

void fp64_launch_iteration(const StepParams& p, int cur, cudaStream_t s, cudaEvent_t* ev) {
    const dim3 blk(SW2D_BX, SW2D_BY);
    if (ev) cudaEventRecord(ev[0], s);
    k64_flux<<<grid_faces(p), blk, 0, s>>>(p, cur);
    if (ev) cudaEventRecord(ev[1], s);
    k64_hstar<<<grid_cells(p), blk, 0, s>>>(p, cur);
    if (ev) cudaEventRecord(ev[2], s);
    k64_depth<<<grid_cells(p), blk, 0, s>>>(p, cur);
    if (ev) cudaEventRecord(ev[3], s);
    k64_facevel<<<grid_faces(p), blk, 0, s>>>(p, cur, 1);
    if (ev) cudaEventRecord(ev[4], s);
}

void fp64_launch_prime(const StepParams& p, int cur, int full, cudaStream_t s) {
    k64_prime<<<grid_cells(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur, full);
}

void fp64_launch_face_velocity(const StepParams& p, int cur, cudaStream_t s) {
    k64_facevel<<<grid_faces(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur, 0);
}

void fp64_launch_cell_velocity(const StepParams& p, int cur, double* uu, double* vv, double* uua,
                               double* vva, cudaStream_t s) {
    k64_cellvel<<<grid_cells(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur, uu, vv, uua, vva);
}

} // namespace sw2d
