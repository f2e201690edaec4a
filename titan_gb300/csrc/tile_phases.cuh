// tile_phases.cuh -- the per-tile arithmetic shared by both step kernels, so
// that the per-tile and the pipelined form give identical bits.
//
// Shared memory holds the tile's state records (tile masses, then halo) in
// the HBM record layout (state.cuh), and one force slot per slab entry:
// FP32 modes a float4 (x, y, z, 0), FP64 two double2 ((x, y), (z, 0)).
//
// Slab entry (spring) force, on the entry's RIGHT end (src/sim.cu:1054-1065):
//   FP64   the reference's operations in the reference's order: |d| with
//          sqrt, d/|d| by division, sin(omega t + phase).
//   FP32*  d = (x_r - x_l) [+ (xl_r - xl_l)], r = 1/|d| from rsqrtf and one
//          Newton step, f = k (rest' - |d|) + c ((v_l - v_r).d) r,
//          F = d (f r); rest' = rest (1 + a sin(2 pi frac(nu T + phi)))
//          with a = -amp for contract-then-expand, +amp otherwise, nu =
//          omega / 2 pi, phi = phase / 2 pi (range-reduced __sinf).
#pragma once

#include "engine.h"
#include "state.cuh"
#include "step_math.cuh"

namespace tg {
namespace {

template <int PREC>
struct Slot {
    static constexpr int kBytes = PREC == P_FP64 ? 32 : 16;  // force slot == entry record size
};

// time of the step in the forms the entry forces use
struct StepTime {
    double T;
    float hi, lo;
};
__device__ __forceinline__ StepTime step_time(double T) {
    StepTime t;
    t.T = T;
    t.hi = (float)T;
    t.lo = (float)(T - (double)t.hi);
    return t;
}

// A slab entry record (FP32: ends, k, rest, damping; FP64: k, rest |
// damping, ends) or an actuation record (FP32: nu, signed amp, phi; FP64:
// omega, amp | phase, -), held by value.
template <int PREC>
struct Rec16 {
    float4 v;
};
template <>
struct Rec16<P_FP64> {
    double2 lo, hi;
};

template <int PREC>
__device__ __forceinline__ Rec16<PREC> load_rec(const uint8_t *p) {  // shared memory
    Rec16<PREC> r;
    if constexpr (PREC == P_FP64) {
        r.lo = reinterpret_cast<const double2 *>(p)[0];
        r.hi = reinterpret_cast<const double2 *>(p)[1];
    } else {
        r.v = *reinterpret_cast<const float4 *>(p);
    }
    return r;
}
template <int PREC>
__device__ __forceinline__ Rec16<PREC> ldg_rec(const uint8_t *p) {  // read-only global memory
    Rec16<PREC> r;
    if constexpr (PREC == P_FP64) {
        r.lo = __ldg(reinterpret_cast<const double2 *>(p));
        r.hi = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    } else {
        r.v = __ldg(reinterpret_cast<const float4 *>(p));
    }
    return r;
}

// The same from a stream read once per step (slab entries, actuation
// records): evict-first in L1 and L2 (ld.global.cs), so that the state
// records, re-read by neighbouring tiles and by the next step, keep L2.
template <int PREC>
__device__ __forceinline__ Rec16<PREC> ldcs_rec(const uint8_t *p) {
    Rec16<PREC> r;
    if constexpr (PREC == P_FP64) {
        r.lo = __ldcs(reinterpret_cast<const double2 *>(p));
        r.hi = __ldcs(reinterpret_cast<const double2 *>(p) + 1);
    } else {
        r.v = __ldcs(reinterpret_cast<const float4 *>(p));
    }
    return r;
}

template <int PREC>
struct F3 {
    typename Real<PREC>::T x, y, z;
};

// Force on the right end of a spring whose ends are the state records sa
// (left) and sb (right) staged at st; k, rest, damping from the spring's
// record, type from its entry word, act its actuation record.
template <int PREC>
__device__ __forceinline__ F3<PREC> spring_force(int sa, int sb, uint32_t type, typename Real<PREC>::T k,
                                                 typename Real<PREC>::T rest, typename Real<PREC>::T damping,
                                                 bool actuated, const Rec16<PREC> &act, const uint8_t *st,
                                                 const StepTime &t) {
    if constexpr (PREC == P_FP64) {
        double scale = 1.0;
        if (actuated) {
            const double2 q01 = act.lo;
            const double2 q23 = act.hi;
            double th = q01.x * t.T;
            th = th + q23.x;
            const double sn = q01.y * sin(th);
            scale = type == 2 ? 1.0 - sn : 1.0 + sn;
        }
        const double2 *pa = reinterpret_cast<const double2 *>(st + (int64_t)sa * 48);
        const double2 *pb = reinterpret_cast<const double2 *>(st + (int64_t)sb * 48);
        const double2 a0 = pa[0], a1 = pa[1], b0 = pb[0], b1 = pb[1];
        const double d0 = b0.x - a0.x, d1 = b0.y - a0.y, d2 = b1.x - a1.x;
        const double nrm = nrm3(d0, d1, d2);
        const double u0 = d0 / nrm, u1 = d1 / nrm, u2 = d2 / nrm;
        const double fs = k * (rest * scale - nrm);
        double f0 = u0 * fs, f1 = u1 * fs, f2 = u2 * fs;
        if (damping != 0.0) {
            const double2 a2 = pa[2], b2 = pb[2];
            const double w0 = a1.y - b1.y, w1 = a2.x - b2.x, w2 = a2.y - b2.y;
            const double dd = ((w0 * u0 + w1 * u1) + w2 * u2) * damping;
            f0 = f0 + u0 * dd;
            f1 = f1 + u1 * dd;
            f2 = f2 + u2 * dd;
        }
        return F3<PREC>{f0, f1, f2};
    } else {
        (void)type;
        float rs = rest;
        if (actuated) {
            const float4 q = act.v;
            const float cyc = fmaf(q.x, t.hi, fmaf(q.x, t.lo, q.z));
            const float fr = cyc - rintf(cyc);
            rs = rest * fmaf(q.y, __sinf(6.28318530717958647692f * fr), 1.0f);
        }
        constexpr int kV = PREC == P_FP32 ? 2 : 3;  // float4 per state record
        const float4 *pa = reinterpret_cast<const float4 *>(st) + sa * kV;
        const float4 *pb = reinterpret_cast<const float4 *>(st) + sb * kV;
        const float4 a0 = pa[0], a1 = pa[1], b0 = pb[0], b1 = pb[1];
        float d0 = b0.x - a0.x, d1 = b0.y - a0.y, d2 = b0.z - a0.z;
        if constexpr (PREC == P_FP32C) {
            const float a2x = pa[2].x, b2x = pb[2].x;
            d0 += b1.z - a1.z;
            d1 += b1.w - a1.w;
            d2 += b2x - a2x;
        }
        const float n2 = fmaf(d2, d2, fmaf(d1, d1, d0 * d0));
        float rq = rsqrtf(n2);
        rq = rq * fmaf(-0.5f * n2 * rq, rq, 1.5f);  // one Newton step
        const float nrm = n2 * rq;
        float f = k * (rs - nrm);
        if (damping != 0.f) {
            const float w0 = a0.w - b0.w, w1 = a1.x - b1.x, w2 = a1.y - b1.y;
            f = fmaf(fmaf(w2, d2, fmaf(w1, d1, w0 * d0)), rq * damping, f);
        }
        const float fr = f * rq;
        return F3<PREC>{d0 * fr, d1 * fr, d2 * fr};
    }
}

// Force of a slab entry (record rec; actuation record act when actuated) on
// its right end, from the state records staged at st; written to slot.
template <int PREC>
__device__ __forceinline__ void entry_force(const Rec16<PREC> &rec, bool actuated, const Rec16<PREC> &act,
                                            const uint8_t *st, const StepTime &t, uint8_t *slot) {
    if constexpr (PREC == P_FP64) {
        const uint32_t ends = (uint32_t)__double_as_longlong(rec.hi.y);
        const F3<PREC> f = spring_force<PREC>(ends & 0xfff, (ends >> 12) & 0xfff, (ends >> 24) & 3, rec.lo.x,
                                              rec.lo.y, rec.hi.x, actuated, act, st, t);
        reinterpret_cast<double2 *>(slot)[0] = make_double2(f.x, f.y);
        reinterpret_cast<double2 *>(slot)[1] = make_double2(f.z, 0.0);
    } else {
        const uint32_t ends = __float_as_uint(rec.v.x);
        const F3<PREC> f = spring_force<PREC>(ends & 0xfff, (ends >> 12) & 0xfff, (ends >> 24) & 3, rec.v.y,
                                              rec.v.z, rec.v.w, actuated, act, st, t);
        *reinterpret_cast<float4 *>(slot) = make_float4(f.x, f.y, f.z, 0.f);
    }
}

// Adds the forces of incidence codes 4w..4w+3 (those below d) of one mass,
// in ascending order: + the slot for a right end, - for a left end.
template <int PREC>
__device__ __forceinline__ void gather_word(const uint8_t *slots, uint2 cw, uint32_t w, uint32_t d,
                                            typename Real<PREC>::T &F0, typename Real<PREC>::T &F1,
                                            typename Real<PREC>::T &F2) {
#pragma unroll
    for (int h = 0; h < 4; h++) {
        if (4 * w + h < d) {
            const uint32_t word = h < 2 ? cw.x : cw.y;
            const uint32_t code = (h & 1) ? (word >> 16) : (word & 0xffffu);
            const int idx = code & 0x7fff;
            if constexpr (PREC == P_FP64) {
                const double sg = (code & 0x8000) ? -1.0 : 1.0;
                const double2 *f = reinterpret_cast<const double2 *>(slots + (int64_t)idx * 32);
                const double2 f01 = f[0], f2v = f[1];
                F0 = fma(sg, f01.x, F0);
                F1 = fma(sg, f01.y, F1);
                F2 = fma(sg, f2v.x, F2);
            } else {
                const float sg = (code & 0x8000) ? -1.0f : 1.0f;
                const float4 f = reinterpret_cast<const float4 *>(slots)[idx];
                F0 = fmaf(sg, f.x, F0);
                F1 = fmaf(sg, f.y, F1);
                F2 = fmaf(sg, f.z, F2);
            }
        }
    }
}

// The same for a whole word: codes past the mass's degree are padding that
// names a slot holding a zero force (+0 adds nothing: the running sum is a
// finite force or +0 after the first code).
template <int PREC>
__device__ __forceinline__ void gather_word_padded(const uint8_t *slots, uint2 cw, typename Real<PREC>::T &F0,
                                                   typename Real<PREC>::T &F1, typename Real<PREC>::T &F2) {
#pragma unroll
    for (int h = 0; h < 4; h++) {
        const uint32_t word = h < 2 ? cw.x : cw.y;
        const uint32_t code = (h & 1) ? (word >> 16) : (word & 0xffffu);
        const int idx = code & 0x7fff;
        if constexpr (PREC == P_FP64) {
            const double sg = (code & 0x8000) ? -1.0 : 1.0;
            const double2 *f = reinterpret_cast<const double2 *>(slots + (int64_t)idx * 32);
            const double2 f01 = f[0], f2v = f[1];
            F0 = fma(sg, f01.x, F0);
            F1 = fma(sg, f01.y, F1);
            F2 = fma(sg, f2v.x, F2);
        } else {
            const float sg = (code & 0x8000) ? -1.0f : 1.0f;
            const float4 f = reinterpret_cast<const float4 *>(slots)[idx];
            F0 = fmaf(sg, f.x, F0);
            F1 = fmaf(sg, f.y, F1);
            F2 = fmaf(sg, f.z, F2);
        }
    }
}

// Warp-cooperative, fixed-order sum over a heavy mass's incidence list
// (lane l takes codes l, l+32, ...; then an xor butterfly).
// warp / nw: this warp's index among the nw warps sharing the work.
template <int PREC>
__device__ __forceinline__ void heavy_sums(const StepArgs &a, const TileInfo &ti, const uint8_t *slots,
                                           typename Real<PREC>::T *sH, int warp, int nw) {
    using R = typename Real<PREC>::T;
    const int lane = threadIdx.x & 31;
    for (int h = warp; h < ti.nheavy; h += nw) {
        const int64_t gh = (int64_t)ti.heavy_off + h;
        const uint32_t q0 = a.heavy_inc_off[gh], q1 = a.heavy_inc_off[gh + 1];
        R p0 = 0, p1 = 0, p2 = 0;
        for (uint32_t q = q0 + lane; q < q1; q += 32) {
            const uint32_t code = a.heavy_inc[q];
            const R *f = reinterpret_cast<const R *>(slots + (int64_t)(code & 0x7fff) * Slot<PREC>::kBytes);
            if (code & 0x8000) {
                p0 = p0 + (-f[0]);
                p1 = p1 + (-f[1]);
                p2 = p2 + (-f[2]);
            } else {
                p0 = p0 + f[0];
                p1 = p1 + f[1];
                p2 = p2 + f[2];
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
            sH[ti.nheavy + h] = p1;
            sH[2 * ti.nheavy + h] = p2;
        }
    }
}

}  // namespace
}  // namespace tg
