// step_math.cuh -- device-side force functions of the step kernels: the
// reference constraint forces in FP64 (reference operation order) and FP32,
// and error-free float transformations for the compensated update.
#pragma once

#include "engine.h"

namespace tg {
namespace {

constexpr double kNormal = 20000.0;  // src/object.cu:26

// ---------------------------------------------------------------- FP64 ----
__device__ __forceinline__ double nrm3(double a, double b, double c) {
    return sqrt((a * a + b * b) + c * c);
}
__device__ __forceinline__ double dot3(const double *a, const double *b) {
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

// src/object.cu:73-106
__device__ __forceinline__ void plane_apply(const double *n, double off, double fk, double fs,
                                            const double *x, const double *v, double *F) {
    double disp = dot3(x, n) - off;
    if (!(disp < 0)) return;  // only zeros would be added otherwise
    double fdn = dot3(F, n);
    double fn[3] = {n[0] * fdn, n[1] * fdn, n[2] * fdn};
    if (fs > 0 || fk > 0) {
        double vdn = dot3(v, n);
        double vp[3] = {v[0] - n[0] * vdn, v[1] - n[1] * vdn, v[2] - n[2] * vdn};
        double vn = nrm3(vp[0], vp[1], vp[2]);
        if (vn > 1e-16) {
            double fmag = fk * nrm3(fn[0], fn[1], fn[2]);
            F[0] = F[0] - (vp[0] * fmag) / vn;
            F[1] = F[1] - (vp[1] * fmag) / vn;
            F[2] = F[2] - (vp[2] * fmag) / vn;
        } else {
            double fp[3] = {F[0] - fn[0], F[1] - fn[1], F[2] - fn[2]};
            if (fs * nrm3(fn[0], fn[1], fn[2]) > nrm3(fp[0], fp[1], fp[2])) {
                F[0] = F[0] - fp[0];
                F[1] = F[1] - fp[1];
                F[2] = F[2] - fp[2];
            }
        }
    }
    double s = (-disp) * kNormal;
    F[0] = F[0] + n[0] * s;
    F[1] = F[1] + n[1] * s;
    F[2] = F[2] + n[2] * s;
}

// src/object.cu:53-56
__device__ __forceinline__ void ball_apply(const double *c, double r, const double *x, double *F) {
    double d[3] = {x[0] - c[0], x[1] - c[1], x[2] - c[2]};
    double dist = nrm3(d[0], d[1], d[2]);
    if (dist <= r) {
        F[0] = F[0] + (kNormal * d[0]) / dist;
        F[1] = F[1] + (kNormal * d[1]) / dist;
        F[2] = F[2] + (kNormal * d[2]) / dist;
    }
}

// src/object.cu:115-124
__device__ __forceinline__ void cplane_apply(const double *n, double fr, double *v, double *F) {
    double nf = dot3(F, n);
    F[0] = F[0] + (-n[0]) * nf;
    F[1] = F[1] + (-n[1]) * nf;
    F[2] = F[2] + (-n[2]) * nf;
    double vn = nrm3(v[0], v[1], v[2]);
    if (vn >= 1e-16) {
        double vdn = dot3(v, n);
        v[0] = v[0] + (-n[0]) * vdn;
        v[1] = v[1] + (-n[1]) * vdn;
        v[2] = v[2] + (-n[2]) * vdn;
        double s = (-fr) * nf;
        F[0] = F[0] + (v[0] * s) / vn;
        F[1] = F[1] + (v[1] * s) / vn;
        F[2] = F[2] + (v[2] * s) / vn;
    }
}

// src/object.cu:133-141
__device__ __forceinline__ void direction_apply(const double *t, double fr, double *v, double *F) {
    double fdt = dot3(F, t);
    double nf[3] = {F[0] - t[0] * fdt, F[1] - t[1] * fdt, F[2] - t[2] * fdt};
    F[0] = F[0] + (-nf[0]);
    F[1] = F[1] + (-nf[1]);
    F[2] = F[2] + (-nf[2]);
    if (nrm3(v[0], v[1], v[2]) >= 1e-16) {
        double vdt = dot3(v, t);
        v[0] = t[0] * vdt;
        v[1] = t[1] * vdt;
        v[2] = t[2] * vdt;
        double s = (-nrm3(nf[0], nf[1], nf[2])) * fr;
        F[0] = F[0] + t[0] * s;
        F[1] = F[1] + t[1] * s;
        F[2] = F[2] + t[2] * s;
    }
}

// Local constraints of one mass (src/sim.cu:1117-1131), records pre-sorted.
__device__ __forceinline__ void local_apply(const StepArgs &a, int64_t g, double *x, double *v,
                                            double *F) {
    for (int32_t r = a.lc_ptr[g]; r < a.lc_ptr[g + 1]; r++) {
        const double *rec = a.lc_rec + 4 * (int64_t)r;
        switch (a.lc_type[r]) {
            case 1: plane_apply(rec, rec[3], 0.0, 0.0, x, v, F); break;
            case 2: ball_apply(rec, rec[3], x, F); break;
            case 0: cplane_apply(rec, rec[3], v, F); break;
            case 3: direction_apply(rec, rec[3], v, F); break;
            default: break;
        }
    }
}

// ---------------------------------------------------------------- FP32 ----
__device__ __forceinline__ float nrm3f(float a, float b, float c) {
    return __fsqrt_rn(fmaf(c, c, fmaf(b, b, a * a)));
}
__device__ __forceinline__ float dot3f(const float *a, const float *b) {
    return fmaf(a[2], b[2], fmaf(a[1], b[1], a[0] * b[0]));
}

__device__ __forceinline__ void plane_applyf(const float *n, float disp, float fk, float fs,
                                             const float *v, float *F) {
    if (!(disp < 0.f)) return;
    float fdn = dot3f(F, n);
    float fn[3] = {n[0] * fdn, n[1] * fdn, n[2] * fdn};
    if (fs > 0.f || fk > 0.f) {
        float vdn = dot3f(v, n);
        float vp[3] = {v[0] - n[0] * vdn, v[1] - n[1] * vdn, v[2] - n[2] * vdn};
        float vn = nrm3f(vp[0], vp[1], vp[2]);
        if (vn > 1e-16f) {
            float fm = __fdiv_rn(fk * nrm3f(fn[0], fn[1], fn[2]), vn);
            F[0] -= vp[0] * fm;
            F[1] -= vp[1] * fm;
            F[2] -= vp[2] * fm;
        } else {
            float fp[3] = {F[0] - fn[0], F[1] - fn[1], F[2] - fn[2]};
            if (fs * nrm3f(fn[0], fn[1], fn[2]) > nrm3f(fp[0], fp[1], fp[2])) {
                F[0] -= fp[0];
                F[1] -= fp[1];
                F[2] -= fp[2];
            }
        }
    }
    float s = (-disp) * 20000.0f;
    F[0] += n[0] * s;
    F[1] += n[1] * s;
    F[2] += n[2] * s;
}

__device__ __forceinline__ void ball_applyf(const float *d, float r, float *F) {
    float dist = nrm3f(d[0], d[1], d[2]);
    if (dist <= r) {
        float s = __fdiv_rn(20000.0f, dist);
        F[0] += d[0] * s;
        F[1] += d[1] * s;
        F[2] += d[2] * s;
    }
}

// error-free transformations (Knuth two-sum, Dekker fast-two-sum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}

// 32-byte record as two read-only 16-byte loads
struct D4 { double x, y, z, w; };
__device__ __forceinline__ D4 ldg_d4(const double *p) {
    double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return D4{a.x, a.y, b.x, b.y};
}

template <int PREC>
struct Real { using T = float; };
template <>
struct Real<P_FP64> { using T = double; };


}  // namespace
}  // namespace tg
