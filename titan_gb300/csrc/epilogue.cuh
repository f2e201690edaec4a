// epilogue.cuh -- the per-mass part of the step, shared by both step kernels:
// gravity, external force, global planes and balls, per-body plane, local
// constraints and drag, then symplectic Euler (src/sim.cu:1100-1166), and the
// store of the new state record.  F0..F2 is the mass's summed spring force;
// s holds its current state (FP32C: hi and lo parts).
#pragma once

#include "engine.h"
#include "state.cuh"
#include "step_math.cuh"

namespace tg {
namespace {

// (hi, lo) += (wh + wl) * (dt_hi + dt_lo) + extra, compensated: the product's
// rounding error and the low parts are carried into lo.
__device__ __forceinline__ void comp_add_prod(float &hi, float &lo, float wh, float wl, float dt_hi, float dt_lo,
                                              float extra) {
    const float q = wh * dt_hi;
    const float qe = fmaf(wh, dt_hi, -q) + fmaf(wh, dt_lo, wl * dt_hi) + extra;
    float sum, err;
    two_sum(hi, q, sum, err);
    err += lo + qe;
    fast_two_sum(sum, err, hi, lo);
}

// INTEG: the integrator (INTEG_*) fixed at compile time, or -1 to read it
// from prm at run time.
template <int PREC, int INTEG = -1>
__device__ __forceinline__ void integrate(const StepArgs &a, const TileInfo &ti, int64_t g, uint8_t fl,
                                          typename Real<PREC>::T m, typename Real<PREC>::T F0,
                                          typename Real<PREC>::T F1, typename Real<PREC>::T F2, St<PREC> &s,
                                          void *out, int64_t gs, int write_acc, int64_t np,
                                          const DevParams *prm) {
    if constexpr (PREC == P_FP64) {
        double Fd[3] = {F0, F1, F2};
        Fd[0] = Fd[0] + prm->g[0] * m;
        Fd[1] = Fd[1] + prm->g[1] * m;
        Fd[2] = Fd[2] + prm->g[2] * m;
        if (fl & MF_EXT) {
            const double *ext = reinterpret_cast<const double *>(a.ext);
            Fd[0] = Fd[0] + ext[g];
            Fd[1] = Fd[1] + ext[np + g];
            Fd[2] = Fd[2] + ext[2 * np + g];
        }
        for (int j = 0; j < prm->nplanes; j++) {
            const double *p = prm->plane[j];
            plane_apply(p, p[3], p[4], p[5], s.x, s.v, Fd);
        }
        for (int j = 0; j < prm->nballs; j++) ball_apply(prm->ball[j], prm->ball[j][3], s.x, Fd);
        if (fl & MF_BODYPLANE) {
            const double *p = a.body_plane + 6 * (int64_t)ti.body;
            plane_apply(p, p[3], p[4], p[5], s.x, s.v, Fd);
        }
        if (fl & MF_LOCAL) local_apply(a, g, s.x, s.v, Fd);
        if (fl & MF_DRAG) {  // src/sim.cu:1134-1137
            double vn = nrm3(s.v[0], s.v[1], s.v[2]);
            if (vn != 0.0) {
                double c = (double)(-a.drag[g]) * (vn * vn);
                Fd[0] = Fd[0] + (s.v[0] * c) / vn;
                Fd[1] = Fd[1] + (s.v[1] * c) / vn;
                Fd[2] = Fd[2] + (s.v[2] * c) / vn;
            }
        }
        const double dt = prm->dt;
        double acc[3] = {Fd[0] / m, Fd[1] / m, Fd[2] / m};
        double *ac = reinterpret_cast<double *>(a.acc);
        const int integ = INTEG >= 0 ? INTEG : prm->integrator;
        if (integ == INTEG_VERLET) {  // src/sim.cu:1155-1159; acc is state
            double ap[3] = {ac[g], ac[np + g], ac[2 * np + g]};
#pragma unroll
            for (int c = 0; c < 3; c++) s.v[c] = s.v[c] + (0.5 * (ap[c] + acc[c])) * dt;
#pragma unroll
            for (int c = 0; c < 3; c++) s.x[c] = s.x[c] + (s.v[c] * dt + (0.5 * acc[c]) * prm->dt2);
            write_acc = 1;
        } else if (integ == INTEG_RK2) {  // src/sim.cu:1141-1154
            if (a.rk2_stage == 0) {
#pragma unroll
                for (int c = 0; c < 3; c++) s.x[c] = s.x[c] + (0.5 * s.v[c]) * dt;
#pragma unroll
                for (int c = 0; c < 3; c++) s.v[c] = s.v[c] + (0.5 * acc[c]) * dt;
            } else {
                // the step's starting state is still this mass's record in
                // the buffer this launch writes
                const St<PREC> b = load_state<PREC>(out, gs);
#pragma unroll
                for (int c = 0; c < 3; c++) s.x[c] = b.x[c] + s.v[c] * dt;
#pragma unroll
                for (int c = 0; c < 3; c++) s.v[c] = b.v[c] + acc[c] * dt;
            }
        } else {  // symplectic Euler, src/sim.cu:1161-1166
#pragma unroll
            for (int c = 0; c < 3; c++) {
                s.v[c] = s.v[c] + acc[c] * dt;
                s.x[c] = s.x[c] + s.v[c] * dt;
            }
        }
        store_state<PREC>(out, gs, s);
        if (write_acc) {
            ac[g] = acc[0];
            ac[np + g] = acc[1];
            ac[2 * np + g] = acc[2];
        }
    } else {
        float Ff[3] = {fmaf(prm->gf[0], m, F0), fmaf(prm->gf[1], m, F1), fmaf(prm->gf[2], m, F2)};
        if (fl & MF_EXT) {
            const float *ext = reinterpret_cast<const float *>(a.ext);
            Ff[0] += ext[g];
            Ff[1] += ext[np + g];
            Ff[2] += ext[2 * np + g];
        }
        float vv[3] = {s.v[0] + s.vl[0], s.v[1] + s.vl[1], s.v[2] + s.vl[2]};
        for (int j = 0; j < prm->nplanes; j++) {
            const float *p = prm->planef[j];
            float disp = (dot3f(s.x, p) - p[3]) + dot3f(s.xl, p);
            plane_applyf(p, disp, p[4], p[5], vv, Ff);
        }
        for (int j = 0; j < prm->nballs; j++) {
            const float *b = prm->ballf[j];
            float dd[3] = {(s.x[0] - b[0]) + s.xl[0], (s.x[1] - b[1]) + s.xl[1], (s.x[2] - b[2]) + s.xl[2]};
            ball_applyf(dd, b[3], Ff);
        }
        if (fl & MF_BODYPLANE) {
            const float *p = a.body_planef + 6 * (int64_t)ti.body;
            float disp = (dot3f(s.x, p) - p[3]) + dot3f(s.xl, p);
            plane_applyf(p, disp, p[4], p[5], vv, Ff);
        }
        if (fl & (MF_LOCAL | MF_DRAG)) {
            // rare paths: evaluate in FP64 on the compensated values
            double x[3], v[3], Fd[3], v0[3];
            for (int c = 0; c < 3; c++) {
                x[c] = (double)s.x[c] + (double)s.xl[c];
                v0[c] = v[c] = (double)s.v[c] + (double)s.vl[c];
                Fd[c] = Ff[c];
            }
            if (fl & MF_LOCAL) local_apply(a, g, x, v, Fd);
            if (fl & MF_DRAG) {
                double vn = nrm3(v[0], v[1], v[2]);
                if (vn != 0.0) {
                    double c = (double)(-a.drag[g]) * (vn * vn);
                    for (int k = 0; k < 3; k++) Fd[k] = Fd[k] + (v[k] * c) / vn;
                }
            }
            for (int c = 0; c < 3; c++) {
                Ff[c] = (float)Fd[c];
                if (v[c] != v0[c]) {  // a constraint projected the velocity
                    s.v[c] = (float)v[c];
                    s.vl[c] = (float)(v[c] - (double)s.v[c]);
                }
            }
        }
        const float inv_m = __frcp_rn(m);
        float acc[3];
        float *ac = reinterpret_cast<float *>(a.acc);
#pragma unroll
        for (int c = 0; c < 3; c++) acc[c] = Ff[c] * inv_m;
        const int integ = INTEG >= 0 ? INTEG : prm->integrator;
        if (integ == INTEG_VERLET) {
            // v += (a_prev + a) dt / 2;  x += v dt + a dt^2 / 2
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const float w = 0.5f * (ac[(int64_t)c * np + g] + acc[c]);
                const float r = (0.5f * acc[c]) * prm->dt2f;
                if constexpr (PREC == P_FP32C) {
                    comp_add_prod(s.v[c], s.vl[c], w, 0.f, prm->dt_hi, prm->dt_lo, 0.f);
                    comp_add_prod(s.x[c], s.xl[c], s.v[c], s.vl[c], prm->dt_hi, prm->dt_lo, r);
                } else {
                    s.v[c] = s.v[c] + w * prm->dt_hi;
                    s.x[c] = s.x[c] + (s.v[c] * prm->dt_hi + r);
                }
            }
            write_acc = 1;
        } else if (integ == INTEG_RK2) {
            if (a.rk2_stage == 0) {
                // x += v dt / 2 (with the step's starting v);  v += a dt / 2
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if constexpr (PREC == P_FP32C) {
                        const float vh = s.v[c], vlo = s.vl[c];
                        comp_add_prod(s.x[c], s.xl[c], 0.5f * vh, 0.5f * vlo, prm->dt_hi, prm->dt_lo, 0.f);
                        comp_add_prod(s.v[c], s.vl[c], 0.5f * acc[c], 0.f, prm->dt_hi, prm->dt_lo, 0.f);
                    } else {
                        s.x[c] = s.x[c] + (0.5f * s.v[c]) * prm->dt_hi;
                        s.v[c] = s.v[c] + (0.5f * acc[c]) * prm->dt_hi;
                    }
                }
            } else {
                // from the step's starting state, still this mass's record in
                // the buffer this launch writes: x = x0 + v dt;  v = v0 + a dt
                const St<PREC> b = load_state<PREC>(out, gs);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    if constexpr (PREC == P_FP32C) {
                        const float vh = s.v[c], vlo = s.vl[c];
                        s.x[c] = b.x[c];
                        s.xl[c] = b.xl[c];
                        comp_add_prod(s.x[c], s.xl[c], vh, vlo, prm->dt_hi, prm->dt_lo, 0.f);
                        s.v[c] = b.v[c];
                        s.vl[c] = b.vl[c];
                        comp_add_prod(s.v[c], s.vl[c], acc[c], 0.f, prm->dt_hi, prm->dt_lo, 0.f);
                    } else {
                        s.x[c] = b.x[c] + s.v[c] * prm->dt_hi;
                        s.v[c] = b.v[c] + acc[c] * prm->dt_hi;
                    }
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if constexpr (PREC == P_FP32C) {
                    // v += a dt with dt = dt_hi + dt_lo, compensated
                    float p = acc[c] * prm->dt_hi;
                    float pe = fmaf(acc[c], prm->dt_hi, -p) + acc[c] * prm->dt_lo;
                    float sum, err;
                    two_sum(s.v[c], p, sum, err);
                    err += s.vl[c] + pe;
                    fast_two_sum(sum, err, s.v[c], s.vl[c]);
                    // x += v dt
                    float q = s.v[c] * prm->dt_hi;
                    float qe = fmaf(s.v[c], prm->dt_hi, -q) + fmaf(s.v[c], prm->dt_lo, s.vl[c] * prm->dt_hi);
                    two_sum(s.x[c], q, sum, err);
                    err += s.xl[c] + qe;
                    fast_two_sum(sum, err, s.x[c], s.xl[c]);
                } else {
                    s.v[c] = s.v[c] + acc[c] * prm->dt_hi;
                    s.x[c] = s.x[c] + s.v[c] * prm->dt_hi;
                }
            }
        }
        store_state<PREC>(out, gs, s);
        if (write_acc) {
            ac[g] = acc[0];
            ac[np + g] = acc[1];
            ac[2 * np + g] = acc[2];
        }
    }
}

// A state record staged in shared memory (same layout as in HBM).
template <int PREC>
__device__ __forceinline__ St<PREC> load_state_smem(const uint8_t *st, int i) {
    St<PREC> s;
    if constexpr (PREC == P_FP64) {
        const double2 *p = reinterpret_cast<const double2 *>(st) + 3 * i;
        const double2 a0 = p[0], a1 = p[1], a2 = p[2];
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a1.x;
        s.v[0] = a1.y; s.v[1] = a2.x; s.v[2] = a2.y;
    } else if constexpr (PREC == P_FP32C) {
        const float4 *p = reinterpret_cast<const float4 *>(st) + 3 * i;
        const float4 a0 = p[0], a1 = p[1], a2 = p[2];
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a0.z;
        s.v[0] = a0.w; s.v[1] = a1.x; s.v[2] = a1.y;
        s.xl[0] = a1.z; s.xl[1] = a1.w; s.xl[2] = a2.x;
        s.vl[0] = a2.y; s.vl[1] = a2.z; s.vl[2] = a2.w;
    } else {
        const float4 *p = reinterpret_cast<const float4 *>(st) + 2 * i;
        const float4 a0 = p[0], a1 = p[1];
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a0.z;
        s.v[0] = a0.w; s.v[1] = a1.x; s.v[2] = a1.y;
        s.xl[0] = s.xl[1] = s.xl[2] = 0.f;
        s.vl[0] = s.vl[1] = s.vl[2] = 0.f;
    }
    return s;
}

}  // namespace
}  // namespace tg
