/* FP64 SW2D step on sm_103a: the plain path whose results match the
 * reference's own kernels (SW2D-EFDC.cu:97-725).
 *
 * GB300's FP64 pipe runs at ~1/64 of the FP32 rate, so this path is bound by
 * FP64 instructions, not HBM.  The step is therefore split so that nothing
 * FP64 is computed twice, in two kernels per iteration:
 *   k64_flux   : new x/y face discharges of every face (flux, :97-353) from the
 *                stored face velocities uu1/vv1 of the previous iteration
 *                (the block's momentum faces packed into a list so that
 *                their binary64 update runs on full warps), and the CFL
 *                face-speed maxima of the entering state
 *   k64_update : per tile, the provisional depth (continuity at t,
 *                :602-664) -> "active and h* < th" flags in shared memory;
 *                treat_error (:695-725, restated per face) and the final
 *                depth at t+dt; the closed faces written back and the face
 *                velocities uu1 = qx/hm, vv1 = qy/hn of the new state
 *                (hm_hn, uu1_vv1, :362-452); FP64 volume / rain / clamp /
 *                outlet sums by block reduction; the last block reduces the
 *                per-block partials in a fixed order and prepares the next
 *                iteration's length and forcing on the device.
 * forward (:670-693) is a buffer swap for the depth (h[cur] -> h[nxt]); the
 * discharges keep fixed roles: qx[0]/qy[0] hold the state, k64_flux writes
 * its new faces into qx[1]/qy[1], and k64_update writes every face, closed
 * or not, back into qx[0]/qy[0] -- so no tile reads a face another tile has
 * already closed (the provisional depth needs them unclosed).
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
            it = sw2d_series_index(time, dts, n);
            r = v[it] + (v[it + 1] - v[it]) / (dts * (time - dts * (it)));
        }
    } else if (mode == 1) {
        it = sw2d_series_index(time, dts, n);
        r = v[it] + (v[it + 1] - v[it]) * ((time - dts * (it)) / dts);
    } else {
        it = sw2d_series_index(time, dts, n);
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
            const int it = sw2d_series_index(time, p.dtoq, p.nq);
            q = Q[(size_t)it * ns + i] + (Q[(size_t)(it + 1) * ns + i] - Q[(size_t)it * ns + i]) /
                                             (p.dtoq * (time - p.dtoq * (it)));
        }
    } else {
        const int it = sw2d_series_index(time, p.dtoq, p.nq);
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
    return sw2d_half(p.mtab[p.mcls[a]] + p.mtab[p.mcls[b]]);
}

/* (g n_f) n_f of the face between cells b and a: the reference's gg*rn*rn
 * (:193, :310), from the class-pair table or the uniform value when the
 * host could evaluate it once with the same operations */
__device__ __forceinline__ double friction_coef(const StepParams& p, size_t b, size_t a) {
    if (!p.mcls) return p.gnn_uni;
    if (p.gnn) return p.gnn[(int)p.mcls[b] * p.ncls + (int)p.mcls[a]];
    const double nf = face_manning(p, b, a);
    return p.g * nf * nf;
}

__device__ __forceinline__ double friction(const StepParams& p, double coef, double sq, double hm) {
    /* :193-198; the division by pow(hm, 1.333333) as a product with hm^-1.333333 */
    if (sw2d_le_pos(hm, p.th)) return 0.00;
    return (coef * sq) * sw2d_rpow_manning(hm);
}

/* a / dx for the continuity: exact scaling when dx is a power of two (the
 * constant-division sequence returns the same bits), else sw2d_div_const */
__device__ __forceinline__ double div_spacing(double a, double d, double rd, int k) {
    if (k < 0) return sw2d_div_const(a, d, rd);
    if (sw2d_is0(a)) return 0.0;
    return k == 0 ? a : sw2d_pow2_down(a, k, rd);
}

/* Upwind donor-cell transport across the edge between two neighbouring
 * faces of the same orientation (the reference's umr/uml, umu/umd, vnr/vnl,
 * vnu/vnd, SW2D-EFDC.cu:171-189, :288-306):
 *     a (q1 + q0) / 2 + |a| (q0 - q1) / 2,   a = (w1 + w0) / 2,
 * with q0 the discharge of the face the edge is read from first.  The
 * reference evaluates every edge twice, once from each face beside it, with
 * the same operands in the same order (+ commutes exactly), so one
 * evaluation per edge gives bit-identical fluxes. */
__device__ __forceinline__ double edge_term(double w1, double w0, double q0, double q1) {
    const double a = sw2d_half(w1 + w0);
    return sw2d_half(a * (q1 + q0)) + sw2d_half(fabs(a) * (q0 - q1));
}

/* Kind of a face (SW2D-EFDC.cu:115-165, same tests in the same order):
 *   0 closed (an inactive side, or both sides at or below th)
 *   1 momentum (gravity, convection, friction)
 *   2 weir from side a, 3 weir from side b (a side's surface below the
 *     other side's bed), 4 dry-bed front (exactly one side above th).
 * Side a is the north (x faces) / west (y faces) cell.  The product
 * (hb - th) (ha - th) < 0 of the reference is decided from the two
 * comparisons with th (the differences keep the comparisons' signs and
 * their product of depths cannot underflow). */
struct FaceK {
    int kind;
    bool wa, wb;
    double ha, hb, za, zb, hha, hhb;
};
__device__ __forceinline__ FaceK classify(bool act, double ha, double hb, const double* __restrict__ z, size_t ia,
                                          size_t ib, double th) {
    FaceK f;
    f.kind = 0;
    f.ha = ha;
    f.hb = hb;
    f.wa = sw2d_gt_pos(ha, th);
    f.wb = sw2d_gt_pos(hb, th);
    f.za = f.zb = f.hha = f.hhb = 0.0;
    if (!act || !(f.wa || f.wb)) return f;
    f.za = z[ia];
    f.zb = z[ib];
    f.hhb = hb + f.zb;
    f.hha = ha + f.za;
    if (sw2d_lt(f.hhb, f.za)) f.kind = 2;
    else if (sw2d_lt(f.hha, f.zb)) f.kind = 3;
    else if ((f.wb && sw2d_lt_pos(ha, th)) || (f.wa && sw2d_lt_pos(hb, th))) f.kind = 4;
    else f.kind = 1;
    return f;
}

/* discharge of a non-momentum face */
__device__ __forceinline__ double face_special(const FaceK& f, double th, double gg) {
    switch (f.kind) {
    case 2: return f.wa ? 0.5440 * f.ha * sw2d_sqrt_rn(gg * f.ha) : 0.0;
    case 3: return f.wb ? -0.544 * f.hb * sw2d_sqrt_rn(gg * f.hb) : 0.0;
    case 4:
        if (sw2d_gt0(f.hb) || sw2d_gt0(f.ha)) {
            const double hhan = (f.hb - th) - (f.ha - th);
            const double sgnm = copysign(1.0, hhan);
            const double hh3 = fmax(f.hhb, f.hha) - fmax(f.zb, f.za);
            return -sgnm * 0.350 * hh3 * sw2d_sqrt_rn(2.00 * gg * hh3);
        }
        return 0.0;
    default: return 0.0;
    }
}

/* momentum update of a face (SW2D-EFDC.cu:165-202 x, :282-319 y): along /
 * across are the face's two edge differences, already scaled. */
__device__ __forceinline__ double face_momentum(const StepParams& p, const FaceK& f, double hm, double q0,
                                                double u0, double vt, double along, double across,
                                                double dt2, double dt2n, size_t ia, size_t ib) {
    const double gg = p.g;
    const double g13 = gg * hm * dt2n * (f.hhb - f.ha - f.za);
    const double sq = sw2d_sqrt_rn(u0 * u0 + vt * vt); /* on the integer pipes, correctly rounded */
    const double ram = friction(p, friction_coef(p, ib, ia), sq, hm);
    const double a = sw2d_half(dt2 * ram);
    /* the division on the integer pipes, correctly rounded (sw2d_div_rn) */
    return sw2d_div_rn((1.00 - a) * q0 + (-along - across - g13), 1.00 + a);
}

__device__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* sm);

/* CFL speed contribution of one face of the entering state: (|velocity| +
 * sqrt(g * mean depth)) / spacing for faces between two active cells whose
 * mean depth is >= th (the oracle's cfl_speed, same operations). */
__device__ __forceinline__ double face_speed(double vel, double hm, double g, double rd) {
    return (fabs(vel) + sw2d_sqrt_rn(g * hm)) * rd;
}

#define NWARP (SW2D_BX * SW2D_BY / 32)

__device__ __forceinline__ int tid_linear() { return threadIdx.y * SW2D_BX + threadIdx.x; }

/* binary32 estimate of a face speed, from integer operations: a conversion
 * from binary64 costs a binary64 operation on this GPU */
__device__ __forceinline__ float face_speed_est(bool ok, double vel, double hm, double g, double rd) {
    return ok ? (fabsf(sw2d_f32_est_of_f64(vel)) + sqrtf(sw2d_f32_est_of_f64(g) * sw2d_f32_est_of_f64(hm))) *
                    sw2d_f32_est_of_f64(rd)
              : 0.0f;
}

/* exact block maxima of the x and the y face speeds together: binary32
 * estimates for every face, binary64 only for the faces within 1e-5 of the
 * block's binary32 maximum; both reductions share their barriers.  The
 * maxima are valid in thread 0. */
__device__ __forceinline__ void block_face_speed_max2(bool okx, double vx, double hmx, double rdx, bool oky,
                                                      double vy, double hmy, double rdy, double g, float* smf,
                                                      unsigned long long* smu, unsigned long long* sx,
                                                      unsigned long long* sy) {
    const int lane = tid_linear() & 31, warp = tid_linear() >> 5;
    const float ex = face_speed_est(okx, vx, hmx, g, rdx), ey = face_speed_est(oky, vy, hmy, g, rdy);
    float mx = ex, my = ey;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        my = fmaxf(my, __shfl_xor_sync(0xffffffffu, my, o));
    }
    if (lane == 0) {
        smf[warp] = mx;
        smf[NWARP + warp] = my;
    }
    __syncthreads();
    mx = smf[0];
    my = smf[NWARP];
#pragma unroll
    for (int k = 1; k < NWARP; k++) {
        mx = fmaxf(mx, smf[k]);
        my = fmaxf(my, smf[NWARP + k]);
    }
    unsigned long long bx = 0ull, by = 0ull;
    if (okx && ex >= mx * 0.99999f) bx = (unsigned long long)__double_as_longlong(face_speed(vx, hmx, g, rdx));
    if (oky && ey >= my * 0.99999f) by = (unsigned long long)__double_as_longlong(face_speed(vy, hmy, g, rdy));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ux = __shfl_down_sync(0xffffffffu, bx, o), uy = __shfl_down_sync(0xffffffffu, by, o);
        bx = ux > bx ? ux : bx;
        by = uy > by ? uy : by;
    }
    if (lane == 0) {
        smu[warp] = bx;
        smu[NWARP + warp] = by;
    }
    __syncthreads();
    if (warp == 0) {
        bx = lane < NWARP ? smu[lane] : 0ull;
        by = lane < NWARP ? smu[NWARP + lane] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ux = __shfl_down_sync(0xffffffffu, bx, o), uy = __shfl_down_sync(0xffffffffu, by, o);
            bx = ux > bx ? ux : bx;
            by = uy > by ? uy : by;
        }
    }
    *sx = bx;
    *sy = by;
}

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY, 3) k64_flux(StepParams p, int cur) {
    __shared__ float smf[2 * SW2D_BX * SW2D_BY / 32];
    __shared__ unsigned long long smu[2 * SW2D_BX * SW2D_BY / 32];
    /* momentum faces of the block, then the edges of the block's cells and of
     * the row above / column left of it */
    __shared__ unsigned char regx[SW2D_BY][SW2D_BX], regy[SW2D_BY][SW2D_BX];
    __shared__ double sea[SW2D_BY + 1][SW2D_BX], sec[SW2D_BY + 1][SW2D_BX];
    __shared__ double seb[SW2D_BY][SW2D_BX + 1], sed[SW2D_BY][SW2D_BX + 1];
    /* the block's momentum faces, packed (thread << 1 | axis), so that the
     * binary64 momentum update runs on full warps whatever the mix of face
     * kinds (weir and dry-bed faces sit among momentum faces on steep thin
     * films); hhb = hb + zb of each momentum face, kept from the
     * classification */
    __shared__ unsigned short mlist[2 * SW2D_BX * SW2D_BY];
    __shared__ double mhhb[2 * SW2D_BX * SW2D_BY];
    __shared__ int mwarp[SW2D_BX * SW2D_BY / 32 + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int c = blockIdx.x * SW2D_BX + tx;
    const int r = blockIdx.y * SW2D_BY + ty;
    const Slot& s = p.clk->slot[cur];
    const bool in = (r <= p.R && c <= p.C);
    const int P = p.P;
    const size_t i = (size_t)(r + H) * P + (c + H);
    const double* __restrict__ h = p.h[cur];
    const double* __restrict__ umo = p.qx[0]; /* the state's discharges */
    const double* __restrict__ vno = p.qy[0];
    const double* __restrict__ uu1 = p.uu1;
    const double* __restrict__ vv1 = p.vv1;
    const double th = p.th;
    /* 1: classify the thread's x face (north of the cell) and y face (west) */
    FaceK fx, fy;
    fx.kind = fy.kind = 0;
    const bool doX = in && s.active && c < p.C, doY = in && s.active && r < p.R;
    const bool edgeS = doX && r == p.R && p.outflow_south;
    if (doX && !edgeS) {
        const uint8_t fe = p.flags[i], fw = p.flags[i - P];
        fx = classify((fe & fw & SW2D_F_ACTIVE) != 0, h[i - P], h[i], p.z, i - P, i, th);
    }
    if (doY) {
        const uint8_t fn = p.flags[i], fs = p.flags[i - 1];
        fy = classify((fn & fs & SW2D_F_ACTIVE) != 0, h[i - 1], h[i], p.z, i - 1, i, th);
    }
    regx[ty][tx] = (unsigned char)(fx.kind == 1);
    regy[ty][tx] = (unsigned char)(fy.kind == 1);
    const int t = ty * SW2D_BX + tx, lane = t & 31, warp = t >> 5;
    if (fx.kind == 1) mhhb[2 * t] = fx.hhb;
    if (fy.kind == 1) mhhb[2 * t + 1] = fy.hhb;
    const unsigned bx = __ballot_sync(0xffffffffu, fx.kind == 1), by = __ballot_sync(0xffffffffu, fy.kind == 1);
    if (lane == 0) mwarp[warp] = __popc(bx) + __popc(by);
    __syncthreads();
    /* 2: each edge once, where a momentum face of the block reads it */
    {
        const bool rx = regx[ty][tx], ry = regy[ty][tx];
        const bool rxS = ty + 1 < SW2D_BY && regx[ty + 1][tx], ryS = ty + 1 < SW2D_BY && regy[ty + 1][tx];
        const bool rxE = tx + 1 < SW2D_BX && regx[ty][tx + 1], ryE = tx + 1 < SW2D_BX && regy[ty][tx + 1];
        sea[ty + 1][tx] = (rx || rxS) ? edge_term(uu1[i + P], uu1[i], umo[i], umo[i + P]) : 0.0;
        seb[ty][tx + 1] = (rx || rxE) ? edge_term(vv1[i + 1], vv1[i - P + 1], umo[i], umo[i + 1]) : 0.0;
        sec[ty + 1][tx] = (ry || ryS) ? edge_term(uu1[i + P], uu1[i + P - 1], vno[i], vno[i + P]) : 0.0;
        sed[ty][tx + 1] = (ry || ryE) ? edge_term(vv1[i + 1], vv1[i], vno[i], vno[i + 1]) : 0.0;
        if (ty == 0) { /* warp 0: the row above, read by the first row's faces */
            const size_t u = i - P;
            sea[0][tx] = rx ? edge_term(uu1[u + P], uu1[u], umo[u], umo[u + P]) : 0.0;
            sec[0][tx] = ry ? edge_term(uu1[u + P], uu1[u + P - 1], vno[u], vno[u + P]) : 0.0;
        } else if (ty == 1 && tx < SW2D_BY) { /* warp 1, eight lanes: the column left */
            const size_t l = (size_t)(blockIdx.y * SW2D_BY + tx + H) * P + (blockIdx.x * SW2D_BX - 1 + H);
            seb[tx][0] = regx[tx][0] ? edge_term(vv1[l + 1], vv1[l - P + 1], umo[l], umo[l + 1]) : 0.0;
            sed[tx][0] = regy[tx][0] ? edge_term(vv1[l + 1], vv1[l], vno[l], vno[l + 1]) : 0.0;
        }
    }
    {
        int base = 0;
        for (int w = 0; w < warp; w++) base += mwarp[w];
        const unsigned lt = (1u << lane) - 1u;
        const int off = base + __popc(bx & lt) + __popc(by & lt);
        if (fx.kind == 1) mlist[off] = (unsigned short)(2 * t);
        if (fy.kind == 1) mlist[off + (fx.kind == 1 ? 1 : 0)] = (unsigned short)(2 * t + 1);
    }
    __syncthreads();
    /* 3: face discharges: the non-momentum faces by their own thread, then
     * the momentum faces from the packed list */
    bool okx = false, oky = false;
    double hmx = 0, hmy = 0, vx = 0, vy = 0;
    if (in) {
        if (s.active) {
            const double gg = p.g;
            /* mean depths of the two faces: the momentum update and the CFL speed */
            const double hmX = (doX && r > 0) ? sw2d_half(h[i] + h[i - P]) : 0.0;
            const double hmY = (doY && c > 0) ? sw2d_half(h[i] + h[i - 1]) : 0.0;
            if (doX) {
                double F;
                if (edgeS) { /* south edge: free overfall when open */
                    const double hw = h[i - P];
                    F = ((p.flags[i - P] & SW2D_F_ACTIVE) && sw2d_gt_pos(hw, th)) ? 0.5440 * hw * sw2d_sqrt_rn(gg * hw)
                                                                                     : 0.0;
                } else {
                    F = face_special(fx, th, gg);
                }
                if (fx.kind != 1) p.qx[1][i] = F;
            }
            if (doY) {
                if (fy.kind != 1) p.qy[1][i] = face_special(fy, th, gg);
            }
            if (p.dt_mode == 1) {
                const uint8_t fc = p.flags[i];
                if (c < p.C && r > 0 && r < p.R && (fc & p.flags[i - P] & SW2D_F_ACTIVE)) {
                    hmx = hmX;
                    okx = sw2d_ge_pos(hmx, th);
                    vx = uu1[i];
                }
                if (r < p.R && c > 0 && c < p.C && (fc & p.flags[i - 1] & SW2D_F_ACTIVE)) {
                    hmy = hmY;
                    oky = sw2d_ge_pos(hmy, th);
                    vy = vv1[i];
                }
            }
        }
    }
    /* the momentum faces, packed: face k of the list is a face of cell
     * (ry, rx) of the block, x (north) or y (west) by its low bit */
    if (s.active) {
        int M = 0;
        for (int w = 0; w < SW2D_BX * SW2D_BY / 32; w++) M += mwarp[w];
        const double dt2 = s.dt2, dt2dx = s.dt2dx, dt2dy = s.dt2dy;
        for (int k = t; k < M; k += SW2D_BX * SW2D_BY) {
            const int id = mlist[k], ft = id >> 1, lx = ft % SW2D_BX, ly = ft / SW2D_BX;
            const int cc = blockIdx.x * SW2D_BX + lx, rr = blockIdx.y * SW2D_BY + ly;
            const size_t j = (size_t)(rr + H) * P + (cc + H);
            FaceK f;
            f.kind = 1;
            f.hhb = mhhb[id];
            if ((id & 1) == 0) { /* x face north of cell j */
                f.ha = h[j - P];
                f.za = p.z[j - P];
                const double hm = sw2d_half(h[j] + h[j - P]);
                const double u11 = dt2dx * (sea[ly + 1][lx] - sea[ly][lx]);
                const double u12 = (cc == 0) ? 0.0 : dt2dy * (seb[ly][lx + 1] - seb[ly][lx]);
                const double vt = sw2d_quarter(vv1[j] + vv1[j + 1] + vv1[j - P] + vv1[j - P + 1]);
                p.qx[1][j] = face_momentum(p, f, hm, umo[j], uu1[j], vt, u11, u12, dt2, dt2dx, j - P, j);
            } else { /* y face west of cell j */
                f.ha = h[j - 1];
                f.za = p.z[j - 1];
                const double hm = sw2d_half(h[j] + h[j - 1]);
                const double v11 = (rr == 0) ? 0.0 : dt2dx * (sec[ly + 1][lx] - sec[ly][lx]);
                const double v12 = dt2dy * (sed[ly][lx + 1] - sed[ly][lx]);
                const double ut = sw2d_quarter(uu1[j] + uu1[j + P] + uu1[j - 1] + uu1[j + P - 1]);
                p.qy[1][j] = face_momentum(p, f, hm, vno[j], vv1[j], ut, v11, v12, dt2, dt2dy, j - 1, j);
            }
        }
    }
    if (p.dt_mode == 1) {
        unsigned long long sx, sy;
        block_face_speed_max2(okx, vx, hmx, p.rdx, oky, vy, hmy, p.rdy, p.g, smf, smu, &sx, &sy);
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
    if (sw2d_gt(ho, p.ev_wl_min)) {
        pct = p.pct_lake;
        evapo = ev;
    } else {
        pct = p.pct_land;
        evapo = 0.000;
    }
    const double rcell = p.rainw ? rr * sw2d_f64_of_f32(p.rainw[i]) : rr; /* exact, off the FP64 pipe */
    /* (((dqx/dx + dqy/dy) - q_src) - r pct) + e; subtracting a zero source
     * and adding a zero evaporation change no value, so they are skipped */
    double sum = div_spacing(divx, p.dx, p.rdx, p.kdx) + div_spacing(divy, p.dy, p.rdy, p.kdy);
    if (f & SW2D_F_SOURCE) {
        double qli = 0.0;
        for (int k = 0; k < p.nsrc; k++)
            if (p.src_idx[k] == (int)i) qli = ql[k];
        sum = sum - qli;
    }
    sum = sum - rcell * pct;
    if (p.evap) sum = sum + evapo;
    double hn = ho - dt2 * sum;
    *raw = hn;
    *rain_term = rcell * pct;
    hn = sw2d_max0(hn);
    if (!(f & SW2D_F_ACTIVE)) hn = 0.00;
    return hn;
}

/* ------------------------------------------------------------------------ */
/* block reductions (fixed order: deterministic for a given grid)            */


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
    if (tid == 0) {
        DevClock* clk = p.clk;
        const Slot& s = clk->slot[cur];
        if (s.active) {
            const double dt2 = s.dt2;
            const double smax = __longlong_as_double((long long)ux) + __longlong_as_double((long long)uy);
            double src = 0.0;
            for (int k = 0; k < p.nsrc; k++) /* a source overridden on its cell adds nothing */
                if (p.src_idx[k] >= 0) src += s.ql2[k];
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
            /* past the iteration limit the next slot is inactive: t_end = t */
            prepare_slot(p, &clk->slot[cur ^ 1], clk->t, clk->s_max,
                         clk->iters < clk->iter_end ? clk->t_end : clk->t);
        } else {
            clk->slot[cur ^ 1] = s;
        }
        clk->counter = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* continuity at t, treat_error, continuity at t+dt, hm_hn + uu1_vv1:         */
/* SW2D-EFDC.cu:602-664, :695-725, :362-452 in one pass                       */

/* Tile of the update kernel: UT_W x UT_H cells (and their north and west
 * faces) per CTA.  The provisional depths ("dry" flags) are evaluated on the
 * tile plus two rows north and west and one row south and east, the new
 * depths on the tile plus the row north and the column west: the faces of
 * the tile read both; the halo is recomputed, not exchanged. */
#define UT_W 64
#define UT_H 16
#define UT_DW (UT_W + 3)
#define UT_DH (UT_H + 3)
#define UT_NW (UT_W + 1)
#define UT_NH (UT_H + 1)

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_update(StepParams p, int cur) {
    __shared__ uint8_t sdry[UT_DH][UT_DW];   /* rows r0-2 .. r0+UT_H, cols c0-2 .. c0+UT_W */
    __shared__ double shn[UT_NH][UT_NW];     /* rows r0-1 .. r0+UT_H-1, cols c0-1 .. c0+UT_W-1 */
    __shared__ double smd[NWARP];
    const int tid = threadIdx.x;
    const int c0 = blockIdx.x * UT_W, r0 = blockIdx.y * UT_H;
    const int nxt = cur ^ 1;
    const Slot& s = p.clk->slot[cur];
    const int P = p.P, R = p.R, C = p.C;
    const double th = p.th;
    const double* __restrict__ fx = p.qx[1]; /* k64_flux's new discharges, read only */
    const double* __restrict__ fy = p.qy[1];
    const double* __restrict__ hc = p.h[cur];
    double vr = 0.0, ve = 0.0, vq = 0.0;
    if (!s.active) {
        /* the loop condition failed: the iteration copies the depth */
        for (int k = tid; k < UT_W * UT_H; k += SW2D_BX * SW2D_BY) {
            const int r = r0 + k / UT_W, c = c0 + k % UT_W;
            if (r < R && c < C) {
                const size_t i = (size_t)(r + H) * P + (c + H);
                p.h[nxt][i] = hc[i];
            }
        }
    } else {
        /* 1: provisional depth at t -> "active and h* < th" (0 outside the raster) */
        for (int k = tid; k < UT_DH * UT_DW; k += SW2D_BX * SW2D_BY) {
            const int rr = k / UT_DW, cc = k - rr * UT_DW;
            const int r = r0 - 2 + rr, c = c0 - 2 + cc;
            uint8_t dflag = 0;
            if (r >= 0 && r < R && c >= 0 && c < C) {
                const size_t i = (size_t)(r + H) * P + (c + H);
                const uint8_t f = p.flags[i];
                double raw, rt;
                const double hs = continuity(p, i, f, hc[i], fx[i + P] - fx[i], fy[i + 1] - fy[i], s.dt2, s.rr1,
                                             s.ev1, s.ql1, &raw, &rt);
                dflag = (uint8_t)((f & SW2D_F_ACTIVE) && sw2d_lt_pos(hs, th));
            }
            sdry[rr][cc] = dflag;
        }
        __syncthreads();
        /* 2: treat_error per face (a face carrying water out of a cell whose
         * provisional depth fell below th is closed, :704-719), final depth
         * at t+dt; written for the tile's own cells, kept in shared memory
         * for the faces */
        for (int k = tid; k < UT_NH * UT_NW; k += SW2D_BX * SW2D_BY) {
            const int rr = k / UT_NW, cc = k - rr * UT_NW;
            const int r = r0 - 1 + rr, c = c0 - 1 + cc;
            double hn = 0.0;
            if (r >= 0 && r < R && c >= 0 && c < C) {
                const size_t i = (size_t)(r + H) * P + (c + H);
                const uint8_t f = p.flags[i];
                const int dr = rr + 1, dc = cc + 1;
                const uint8_t dC = sdry[dr][dc];
                double fN = fx[i], fS = fx[i + P], fW = fy[i], fE = fy[i + 1];
                if ((sw2d_gt0(fN) && sdry[dr - 1][dc]) || (sw2d_lt0(fN) && dC)) fN = 0;
                if ((sw2d_gt0(fS) && dC) || (sw2d_lt0(fS) && sdry[dr + 1][dc])) fS = 0;
                if ((sw2d_gt0(fW) && sdry[dr][dc - 1]) || (sw2d_lt0(fW) && dC)) fW = 0;
                if ((sw2d_gt0(fE) && dC) || (sw2d_lt0(fE) && sdry[dr][dc + 1])) fE = 0;
                const double ho = hc[i];
                double raw, rt;
                hn = continuity(p, i, f, ho, fS - fN, fE - fW, s.dt2, s.rr2, s.ev2, s.ql2, &raw, &rt);
                if (rr >= 1 && cc >= 1) { /* the tile's own cell */
                    p.h[nxt][i] = hn;
                    if (f & SW2D_F_ACTIVE) {
                        if (sw2d_lt0(raw)) atomicAdd(&p.clk->led[LED_CLAMP], -raw * p.area); /* max(h, 0) gain */
                        if (p.ledger_cells) {
                            vr += rt;
                            ve += sw2d_gt(ho, p.ev_wl_min) ? s.ev2 : 0.0;
                        }
                        if (r == R - 1) vq += fS;
                    }
                }
            }
            shn[rr][cc] = hn;
        }
        __syncthreads();
        /* 3: the closed faces written back and the face velocities of the new
         * state, uu1 = qx/hm and vv1 = qy/hn (hm_hn, uu1_vv1), for the
         * tile's north and west faces (the raster's south and east edge
         * faces in the last tile row / column) */
        for (int k = tid; k < UT_H * UT_W; k += SW2D_BX * SW2D_BY) {
            const int rr = k / UT_W, cc = k - rr * UT_W;
            const int r = r0 + rr, c = c0 + cc;
            if (r > R || c > C) continue;
            const size_t i = (size_t)(r + H) * P + (c + H);
            const int dr = rr + 2, dc = cc + 2, nr = rr + 1, nc = cc + 1;
            if (c < C) {
                double F = fx[i];
                if ((sw2d_gt0(F) && sdry[dr - 1][dc]) || (sw2d_lt0(F) && sdry[dr][dc])) F = 0;
                p.qx[0][i] = F;
                double hm;
                if (r == 0) hm = shn[nr][nc];
                else if (r == R) hm = shn[nr - 1][nc];
                else hm = sw2d_half(shn[nr][nc] + shn[nr - 1][nc]);
                p.uu1[i] = sw2d_ge_pos(hm, th) ? (sw2d_is0(F) ? F : sw2d_div_rn(F, hm)) : 0.00; /* 0/hm is 0 of F's sign */
            }
            if (r < R) {
                double F = fy[i];
                if ((sw2d_gt0(F) && sdry[dr][dc - 1]) || (sw2d_lt0(F) && sdry[dr][dc])) F = 0;
                p.qy[0][i] = F;
                double hn;
                if (c == 0) hn = shn[nr][nc];
                else if (c == C) hn = shn[nr][nc - 1];
                else hn = sw2d_half(shn[nr][nc] + shn[nr][nc - 1]);
                p.vv1[i] = sw2d_ge_pos(hn, th) ? (sw2d_is0(F) ? F : sw2d_div_rn(F, hn)) : 0.0;
            }
        }
    }
    /* ledger partials of the tile, then the last block's reduction */
    double pr = 0.0, pe = 0.0, pq = 0.0;
    if (p.ledger_cells) {
        pr = block_sum(vr, smd);
        pe = block_sum(ve, smd);
    }
    if (p.outflow_south) pq = block_sum(vq, smd);
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
    __shared__ float smf[2 * NWARP];
    __shared__ unsigned long long smu[2 * NWARP];
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
    unsigned long long sx, sy;
    block_face_speed_max2(okx, vx, hmx, p.rdx, oky, vy, hmy, p.rdy, p.g, smf, smu, &sx, &sy);
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
        if (full != 1)
            prepare_slot(p, &clk->slot[cur], clk->t, clk->s_max, clk->iters < clk->iter_end ? clk->t_end : clk->t);
        clk->counter = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* hm_hn + uu1_vv1: SW2D-EFDC.cu:362-452, the face velocities of the current
 * state (after its depth was set or restored; the iteration's own are
 * written by k64_update) */

__global__ void __launch_bounds__(SW2D_BX * SW2D_BY) k64_facevel(StepParams p, int cur) {
    const int c = blockIdx.x * SW2D_BX + threadIdx.x;
    const int r = blockIdx.y * SW2D_BY + threadIdx.y;
    if (r > p.R || c > p.C) return;
    const int P = p.P;
    const size_t i = (size_t)(r + H) * P + (c + H);
    const double* __restrict__ h = p.h[cur];
    const double th = p.th;
    if (c < p.C) {
        const double F = p.qx[0][i];
        double hm;
        if (r == 0) hm = h[i];
        else if (r == p.R) hm = h[i - P];
        else hm = sw2d_half(h[i] + h[i - P]);
        p.uu1[i] = sw2d_ge_pos(hm, th) ? (sw2d_is0(F) ? F : sw2d_div_rn(F, hm)) : 0.00; /* 0/hm is 0 of F's sign */
    }
    if (r < p.R) {
        const double F = p.qy[0][i];
        double hn;
        if (c == 0) hn = h[i];
        else if (c == p.C) hn = h[i - 1];
        else hn = sw2d_half(h[i] + h[i - 1]);
        p.vv1[i] = sw2d_ge_pos(hn, th) ? (sw2d_is0(F) ? F : sw2d_div_rn(F, hn)) : 0.0;
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

int fp64_kernels_per_iteration() { return 2; }

void fp64_launch_iteration(const StepParams& p, int cur, cudaStream_t s, cudaEvent_t* ev) {
    const dim3 blk(SW2D_BX, SW2D_BY);
    if (ev) cudaEventRecord(ev[0], s);
    k64_flux<<<grid_faces(p), blk, 0, s>>>(p, cur);
    if (ev) cudaEventRecord(ev[1], s);
    const dim3 gu((p.C + 1 + UT_W - 1) / UT_W, (p.R + 1 + UT_H - 1) / UT_H);
    k64_update<<<gu, SW2D_BX * SW2D_BY, 0, s>>>(p, cur);
    if (ev) cudaEventRecord(ev[2], s);
}

void fp64_launch_prime(const StepParams& p, int cur, int full, cudaStream_t s) {
    k64_prime<<<grid_cells(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur, full);
}

void fp64_launch_face_velocity(const StepParams& p, int cur, cudaStream_t s) {
    k64_facevel<<<grid_faces(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur);
}

void fp64_launch_cell_velocity(const StepParams& p, int cur, double* uu, double* vv, double* uua,
                               double* vva, cudaStream_t s) {
    k64_cellvel<<<grid_cells(p), dim3(SW2D_BX, SW2D_BY), 0, s>>>(p, cur, uu, vv, uua, vva);
}

} // namespace sw2d
