// step.cu -- fused mass-spring step for sm_103a.
//
// One CTA per tile (plan.h).  Per step and tile:
//   A. stage the tile's masses and its halo (positions, velocities) in shared
//      memory;
//   B. compute every slab entry's spring force once (src/sim.cu:1054-1065)
//      into shared memory;
//   C. per mass, sum its incident entries in ascending spring order (the
//      order of one legal serialisation of the reference's atomics,
//      src/vec.cu:33-37), then gravity, external force, global planes and
//      balls, local constraints, drag and the symplectic Euler update
//      (src/sim.cu:1100-1166), and write the other ping-pong buffer.
// The FP64 form is compiled without FMA contraction (build flag --fmad=false)
// so that each operation is rounded as in the CPU oracle.
#include "engine.h"

#include <cstdint>
#include <type_traits>

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

// ------------------------------------------------------------- kernel -----
template <int PREC>
__global__ void __launch_bounds__(512) k_step(StepArgs a, int parity, int write_acc) {
    using R = typename Real<PREC>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileInfo ti = a.tiles[blockIdx.x];
    const int S = a.slots, E = a.ecap;
    R *sx = reinterpret_cast<R *>(smem_raw);  // 3*S positions (hi)
    R *sv = sx + 3 * S;                        // 3*S velocities (hi)
    R *sxl = sv + 3 * S;                       // 3*S position lo (FP32C only)
    R *sF = (PREC == P_FP32C) ? sxl + 3 * S : sxl;  // 3*E entry forces
    R *sH = sF + 3 * E;                        // 3*hcap heavy-mass sums
    const R *in = reinterpret_cast<const R *>(parity ? a.state1 : a.state0);
    R *out = reinterpret_cast<R *>(parity ? a.state0 : a.state1);
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const double T = a.tbuf[parity];
    if (blockIdx.x == 0 && threadIdx.x == 0) a.tbuf[parity ^ 1] = T + prm->dt;

    // ---- A: stage tile + halo -------------------------------------------
    for (int i = threadIdx.x; i < ti.nm + ti.nh; i += blockDim.x) {
        int64_t g = i < ti.nm ? (int64_t)ti.mass_off + i : (int64_t)a.halo[ti.halo_off + i - ti.nm];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            sx[c * S + i] = in[c * np + g];
            sv[c * S + i] = in[(3 + c) * np + g];
            if (PREC == P_FP32C) sxl[c * S + i] = in[(6 + c) * np + g];
        }
    }
    __syncthreads();

    // ---- B: one force per slab entry --------------------------------------
    if constexpr (PREC == P_FP64) {
        const double *ent = reinterpret_cast<const double *>(a.ent) + 4 * (int64_t)ti.ent_off;
        const double *act = reinterpret_cast<const double *>(a.act) + 4 * (int64_t)ti.ent_off;
        for (int e = threadIdx.x; e < ti.ne; e += blockDim.x) {
            D4 r = ldg_d4(ent + 4 * e);
            uint32_t ends = (uint32_t)__double_as_longlong(r.w);
            int sa = ends & 0xfff, sb = (ends >> 12) & 0xfff;
            double scale = 1.0;
            if (e < ti.nact) {
                D4 q = ldg_d4(act + 4 * e);
                double th = q.x * T;
                th = th + q.z;
                double s = q.y * sin(th);
                scale = ((ends >> 24) & 3) == 2 ? 1.0 - s : 1.0 + s;
            }
            double d0 = sx[sb] - sx[sa], d1 = sx[S + sb] - sx[S + sa], d2 = sx[2 * S + sb] - sx[2 * S + sa];
            double nrm = nrm3(d0, d1, d2);
            double u0 = d0 / nrm, u1 = d1 / nrm, u2 = d2 / nrm;
            double fs = r.x * (r.y * scale - nrm);
            double f0 = u0 * fs, f1 = u1 * fs, f2 = u2 * fs;
            if (r.z != 0.0) {
                double w0 = sv[sa] - sv[sb], w1 = sv[S + sa] - sv[S + sb], w2 = sv[2 * S + sa] - sv[2 * S + sb];
                double dd = ((w0 * u0 + w1 * u1) + w2 * u2) * r.z;
                f0 = f0 + u0 * dd;
                f1 = f1 + u1 * dd;
                f2 = f2 + u2 * dd;
            }
            sF[e] = f0;
            sF[E + e] = f1;
            sF[2 * E + e] = f2;
        }
    } else {
        const float4 *ent = reinterpret_cast<const float4 *>(a.ent) + ti.ent_off;
        const float4 *act = reinterpret_cast<const float4 *>(a.act) + ti.ent_off;
        const float Thi = (float)T;
        const float Tlo = (float)(T - (double)Thi);
        for (int e = threadIdx.x; e < ti.ne; e += blockDim.x) {
            float4 r = __ldg(ent + e);
            uint32_t ends = __float_as_uint(r.x);
            int sa = ends & 0xfff, sb = (ends >> 12) & 0xfff;
            float rs = r.z;
            if (e < ti.nact) {
                float4 q = __ldg(act + e);
                float th = fmaf(q.x, Thi, fmaf(q.x, Tlo, q.z));
                float s = q.y * sinf(th);
                rs = r.z * (((ends >> 24) & 3) == 2 ? 1.0f - s : 1.0f + s);
            }
            float d0 = sx[sb] - sx[sa], d1 = sx[S + sb] - sx[S + sa], d2 = sx[2 * S + sb] - sx[2 * S + sa];
            if (PREC == P_FP32C) {
                d0 += sxl[sb] - sxl[sa];
                d1 += sxl[S + sb] - sxl[S + sa];
                d2 += sxl[2 * S + sb] - sxl[2 * S + sa];
            }
            float nrm = nrm3f(d0, d1, d2);
            float inv = __frcp_rn(nrm);
            float u0 = d0 * inv, u1 = d1 * inv, u2 = d2 * inv;
            float f = r.y * (rs - nrm);
            if (r.w != 0.f) {
                float w0 = sv[sa] - sv[sb], w1 = sv[S + sa] - sv[S + sb], w2 = sv[2 * S + sa] - sv[2 * S + sb];
                f = fmaf(fmaf(w2, u2, fmaf(w1, u1, w0 * u0)), r.w, f);
            }
            sF[e] = u0 * f;
            sF[E + e] = u1 * f;
            sF[2 * E + e] = u2 * f;
        }
    }
    __syncthreads();

    // ---- C0: warp-cooperative sums for heavy masses -----------------------
    if (ti.nheavy > 0) {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int h = warp; h < ti.nheavy; h += nw) {
            const int64_t gh = (int64_t)ti.heavy_off + h;
            const uint32_t q0 = a.heavy_inc_off[gh], q1 = a.heavy_inc_off[gh + 1];
            R p0 = 0, p1 = 0, p2 = 0;
            for (uint32_t q = q0 + lane; q < q1; q += 32) {
                uint32_t code = a.heavy_inc[q];
                int idx = code & 0x7fff;
                if (code & 0x8000) {
                    p0 = p0 + (-sF[idx]);
                    p1 = p1 + (-sF[E + idx]);
                    p2 = p2 + (-sF[2 * E + idx]);
                } else {
                    p0 = p0 + sF[idx];
                    p1 = p1 + sF[E + idx];
                    p2 = p2 + sF[2 * E + idx];
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) {
                p0 = p0 + __shfl_xor_sync(0xffffffffu, p0, off);
                p1 = p1 + __shfl_xor_sync(0xffffffffu, p1, off);
                p2 = p2 + __shfl_xor_sync(0xffffffffu, p2, off);
            }
            if (lane == 0) {
                sH[h] = p0;
                sH[a.hcap + h] = p1;
                sH[2 * a.hcap + h] = p2;
            }
        }
        __syncthreads();
    }

    // ---- C: per-mass gather, constraints, integration ----------------------
    for (int i = threadIdx.x; i < ti.nm; i += blockDim.x) {
        const int64_t g = (int64_t)ti.mass_off + i;
        const uint8_t fl = a.flags[g];
        if (fl & MF_FIXED) continue;  // src/sim.cu:1100
        const uint32_t d = a.deg[g];
        R F[3] = {0, 0, 0};
        if (d == 255) {
            int h = 0;
            while (h < ti.nheavy && a.heavy_local[ti.heavy_off + h] != i) h++;
            F[0] = F[0] + sH[h];
            F[1] = F[1] + sH[a.hcap + h];
            F[2] = F[2] + sH[2 * a.hcap + h];
        } else if (d > 0) {
            const uint16_t *ip = a.inc + a.warp_inc_off[ti.warp_off + (i >> 5)] + (i & 31);
            for (uint32_t j = 0; j < d; j++) {
                uint32_t code = __ldg(ip + 32 * j);
                int idx = code & 0x7fff;
                if (code & 0x8000) {
                    F[0] = F[0] + (-sF[idx]);
                    F[1] = F[1] + (-sF[E + idx]);
                    F[2] = F[2] + (-sF[2 * E + idx]);
                } else {
                    F[0] = F[0] + sF[idx];
                    F[1] = F[1] + sF[E + idx];
                    F[2] = F[2] + sF[2 * E + idx];
                }
            }
        }
        if constexpr (PREC == P_FP64) {
            const double m = reinterpret_cast<const double *>(a.mass)[g];
            double x[3] = {sx[i], sx[S + i], sx[2 * S + i]};
            double v[3] = {sv[i], sv[S + i], sv[2 * S + i]};
            double *Fd = reinterpret_cast<double *>(F);
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
                plane_apply(p, p[3], p[4], p[5], x, v, Fd);
            }
            for (int j = 0; j < prm->nballs; j++) ball_apply(prm->ball[j], prm->ball[j][3], x, Fd);
            if (fl & MF_BODYPLANE) {
                const double *p = a.body_plane + 6 * (int64_t)ti.body;
                plane_apply(p, p[3], p[4], p[5], x, v, Fd);
            }
            if (fl & MF_LOCAL) local_apply(a, g, x, v, Fd);
            if (fl & MF_DRAG) {  // src/sim.cu:1134-1137
                double vn = nrm3(v[0], v[1], v[2]);
                if (vn != 0.0) {
                    double c = (double)(-a.drag[g]) * (vn * vn);
                    Fd[0] = Fd[0] + (v[0] * c) / vn;
                    Fd[1] = Fd[1] + (v[1] * c) / vn;
                    Fd[2] = Fd[2] + (v[2] * c) / vn;
                }
            }
            const double dt = prm->dt;
            double acc[3] = {Fd[0] / m, Fd[1] / m, Fd[2] / m};
            double *o = reinterpret_cast<double *>(out);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                v[c] = v[c] + acc[c] * dt;
                x[c] = x[c] + v[c] * dt;
                o[c * np + g] = x[c];
                o[(3 + c) * np + g] = v[c];
            }
            if (write_acc) {
                double *ac = reinterpret_cast<double *>(a.acc);
                ac[g] = acc[0];
                ac[np + g] = acc[1];
                ac[2 * np + g] = acc[2];
            }
        } else {
            float *Ff = reinterpret_cast<float *>(F);
            const float m = reinterpret_cast<const float *>(a.mass)[g];
            float xh[3] = {(float)sx[i], (float)sx[S + i], (float)sx[2 * S + i]};
            float xl[3] = {0.f, 0.f, 0.f};
            float vh[3] = {(float)sv[i], (float)sv[S + i], (float)sv[2 * S + i]};
            float vl[3] = {0.f, 0.f, 0.f};
            const float *inf = reinterpret_cast<const float *>(in);
            if (PREC == P_FP32C) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    xl[c] = (float)sxl[c * S + i];
                    vl[c] = inf[(9 + c) * np + g];
                }
            }
            Ff[0] = fmaf(prm->gf[0], m, Ff[0]);
            Ff[1] = fmaf(prm->gf[1], m, Ff[1]);
            Ff[2] = fmaf(prm->gf[2], m, Ff[2]);
            if (fl & MF_EXT) {
                const float *ext = reinterpret_cast<const float *>(a.ext);
                Ff[0] += ext[g];
                Ff[1] += ext[np + g];
                Ff[2] += ext[2 * np + g];
            }
            float vv[3] = {vh[0] + vl[0], vh[1] + vl[1], vh[2] + vl[2]};
            for (int j = 0; j < prm->nplanes; j++) {
                const float *p = prm->planef[j];
                float disp = (dot3f(xh, p) - p[3]) + dot3f(xl, p);
                plane_applyf(p, disp, p[4], p[5], vv, Ff);
            }
            for (int j = 0; j < prm->nballs; j++) {
                const float *b = prm->ballf[j];
                float dd[3] = {(xh[0] - b[0]) + xl[0], (xh[1] - b[1]) + xl[1], (xh[2] - b[2]) + xl[2]};
                ball_applyf(dd, b[3], Ff);
            }
            if (fl & MF_BODYPLANE) {
                const float *p = a.body_planef + 6 * (int64_t)ti.body;
                float disp = (dot3f(xh, p) - p[3]) + dot3f(xl, p);
                plane_applyf(p, disp, p[4], p[5], vv, Ff);
            }
            if (fl & (MF_LOCAL | MF_DRAG)) {
                // rare paths: evaluate in FP64 on the compensated values
                double x[3], v[3], Fd[3];
                for (int c = 0; c < 3; c++) {
                    x[c] = (double)xh[c] + (double)xl[c];
                    v[c] = (double)vh[c] + (double)vl[c];
                    Fd[c] = Ff[c];
                }
                double v0[3] = {v[0], v[1], v[2]};
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
                        vh[c] = (float)v[c];
                        vl[c] = (float)(v[c] - (double)vh[c]);
                    }
                }
            }
            const float inv_m = __frcp_rn(m);
            float acc[3];
            float *o = reinterpret_cast<float *>(out);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                acc[c] = Ff[c] * inv_m;
                if (PREC == P_FP32C) {
                    // v += a dt with dt = dt_hi + dt_lo, compensated
                    float p = acc[c] * prm->dt_hi;
                    float pe = fmaf(acc[c], prm->dt_hi, -p) + acc[c] * prm->dt_lo;
                    float s, e;
                    two_sum(vh[c], p, s, e);
                    e += vl[c] + pe;
                    fast_two_sum(s, e, vh[c], vl[c]);
                    // x += v dt
                    float q = vh[c] * prm->dt_hi;
                    float qe = fmaf(vh[c], prm->dt_hi, -q) + fmaf(vh[c], prm->dt_lo, vl[c] * prm->dt_hi);
                    two_sum(xh[c], q, s, e);
                    e += xl[c] + qe;
                    fast_two_sum(s, e, xh[c], xl[c]);
                    o[c * np + g] = xh[c];
                    o[(3 + c) * np + g] = vh[c];
                    o[(6 + c) * np + g] = xl[c];
                    o[(9 + c) * np + g] = vl[c];
                } else {
                    vh[c] = vh[c] + acc[c] * prm->dt_hi;
                    xh[c] = xh[c] + vh[c] * prm->dt_hi;
                    o[c * np + g] = xh[c];
                    o[(3 + c) * np + g] = vh[c];
                }
            }
            if (write_acc) {
                float *ac = reinterpret_cast<float *>(a.acc);
                ac[g] = acc[0];
                ac[np + g] = acc[1];
                ac[2 * np + g] = acc[2];
            }
        }
    }
}

// ------------------------------------------------- gather / scatter -------
template <int PREC>
__global__ void k_gather(XferArgs a) {
    using R = typename Real<PREC>::T;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    int64_t src = a.idx ? a.idx[i] : i;
    int64_t g = a.old2new[src];
    const R *st = reinterpret_cast<const R *>(a.parity ? a.state1 : a.state0);
    const int64_t np = a.npad;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double x = (double)st[c * np + g], v = (double)st[(3 + c) * np + g];
        if (PREC == P_FP32C) {
            x += (double)st[(6 + c) * np + g];
            v += (double)st[(9 + c) * np + g];
        }
        if (a.pos) a.pos[3 * i + c] = x;
        if (a.vel) a.vel[3 * i + c] = v;
        if (a.accout) a.accout[3 * i + c] = (double)reinterpret_cast<const R *>(a.acc)[c * np + g];
    }
}

template <int PREC>
__global__ void k_scatter(XferArgs a) {
    using R = typename Real<PREC>::T;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    int64_t src = a.idx ? a.idx[i] : i;
    int64_t g = a.old2new[src];
    const int64_t np = a.npad;
    R *bufs[2] = {reinterpret_cast<R *>(a.state0), reinterpret_cast<R *>(a.state1)};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        for (int b = 0; b < 2; b++) {
            R *st = bufs[b];
            if (a.ipos) {
                double x = a.ipos[3 * i + c];
                R h = (R)x;
                st[c * np + g] = h;
                if (PREC == P_FP32C) st[(6 + c) * np + g] = (R)(x - (double)h);
            }
            if (a.ivel) {
                double v = a.ivel[3 * i + c];
                R h = (R)v;
                st[(3 + c) * np + g] = h;
                if (PREC == P_FP32C) st[(9 + c) * np + g] = (R)(v - (double)h);
            }
        }
        if (a.ipos) reinterpret_cast<R *>(a.acc)[c * np + g] = (R)0;
    }
}

// ------------------------------------------------------ diagnostics -------
// Pass 1: each of kDiagBlocks blocks sums a fixed grid-stride share in FP64
// and reduces it with a fixed tree; pass 2 reduces the partials the same way.
template <int PREC>
__global__ void __launch_bounds__(256) k_diag1(DiagArgs a) {
    using R = typename Real<PREC>::T;
    __shared__ double red[kDiagQ][256];
    double q[kDiagQ];
#pragma unroll
    for (int k = 0; k < kDiagQ; k++) q[k] = 0.0;
    const R *st = reinterpret_cast<const R *>(a.state);
    const R *ms = reinterpret_cast<const R *>(a.mass);
    const int64_t np = a.npad;
    auto pos = [&](int64_t g, int c) {
        double x = (double)st[c * np + g];
        if (PREC == P_FP32C) x += (double)st[(6 + c) * np + g];
        return x;
    };
    auto vel = [&](int64_t g, int c) {
        double v = (double)st[(3 + c) * np + g];
        if (PREC == P_FP32C) v += (double)st[(9 + c) * np + g];
        return v;
    };
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.n; g += stride) {
        double m = (double)ms[g];
        double x[3] = {pos(g, 0), pos(g, 1), pos(g, 2)};
        double v[3] = {vel(g, 0), vel(g, 1), vel(g, 2)};
        double vn = nrm3(v[0], v[1], v[2]);
        q[1] += (0.5 * m) * (vn * vn);
        q[2] += (a.g_mag * x[2]) * m;
        double p[3] = {v[0] * m, v[1] * m, v[2] * m};
        q[3] += p[0];
        q[4] += p[1];
        q[5] += p[2];
        q[6] += p[1] * x[2] - p[2] * x[1];
        q[7] += x[0] * p[2] - p[0] * x[2];
        q[8] += p[0] * x[1] - p[1] * x[0];
    }
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < a.ns; s += stride) {
        int32_t l = a.sl[s], r = a.sr[s];
        if (l < 0) continue;
        double d0 = pos(l, 0) - pos(r, 0), d1 = pos(l, 1) - pos(r, 1), d2 = pos(l, 2) - pos(r, 2);
        double x = nrm3(d0, d1, d2) - a.srest[s];
        q[0] += (a.sk[s] * (x * x)) / 2;
    }
#pragma unroll
    for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] = q[k];
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) a.partials[blockIdx.x * kDiagQ + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) k_diag2(DiagArgs a) {
    __shared__ double red[kDiagQ][256];
    for (int k = 0; k < kDiagQ; k++) {
        double s = 0.0;
        for (int b = threadIdx.x; b < kDiagBlocks; b += 256) s += a.partials[b * kDiagQ + k];
        red[k][threadIdx.x] = s;
    }
    __syncthreads();
    for (int w = 128; w >= 1; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int k = 0; k < kDiagQ; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) a.out[threadIdx.x] = red[threadIdx.x][0];
}

}  // namespace

size_t step_smem_bytes(int precision, int slots, int ecap, int hcap) {
    size_t words = (size_t)(precision == P_FP32C ? 9 : 6) * slots + 3 * (size_t)ecap + 3 * (size_t)hcap;
    return words * (precision == P_FP64 ? sizeof(double) : sizeof(float));
}

cudaError_t step_prepare(int precision, size_t smem) {
    const void *f = precision == P_FP64   ? (const void *)k_step<P_FP64>
                    : precision == P_FP32 ? (const void *)k_step<P_FP32>
                                          : (const void *)k_step<P_FP32C>;
    return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_step(int precision, const StepArgs &a, int ntiles, int threads, size_t smem,
                        int parity, int write_acc, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    switch (precision) {
        case P_FP64: k_step<P_FP64><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
        case P_FP32: k_step<P_FP32><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
        default: k_step<P_FP32C><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_gather(int precision, const XferArgs &a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    int blocks = (int)((a.count + 255) / 256);
    switch (precision) {
        case P_FP64: k_gather<P_FP64><<<blocks, 256, 0, s>>>(a); break;
        case P_FP32: k_gather<P_FP32><<<blocks, 256, 0, s>>>(a); break;
        default: k_gather<P_FP32C><<<blocks, 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_scatter(int precision, const XferArgs &a, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    int blocks = (int)((a.count + 255) / 256);
    switch (precision) {
        case P_FP64: k_scatter<P_FP64><<<blocks, 256, 0, s>>>(a); break;
        case P_FP32: k_scatter<P_FP32><<<blocks, 256, 0, s>>>(a); break;
        default: k_scatter<P_FP32C><<<blocks, 256, 0, s>>>(a); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_diag(int precision, const DiagArgs &a, cudaStream_t s) {
    switch (precision) {
        case P_FP64: k_diag1<P_FP64><<<kDiagBlocks, 256, 0, s>>>(a); break;
        case P_FP32: k_diag1<P_FP32><<<kDiagBlocks, 256, 0, s>>>(a); break;
        default: k_diag1<P_FP32C><<<kDiagBlocks, 256, 0, s>>>(a); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_diag2<<<1, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace tg
