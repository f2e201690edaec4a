// state.cuh -- one mass's state record in HBM (tiled order), moved with 16-byte
// vectors:
//   FP64  48 B: x0 x1 | x2 v0 | v1 v2                               (3 x double2)
//   FP32C 48 B: xh0 xh1 xh2 vh0 | vh1 vh2 xl0 xl1 | xl2 vl0 vl1 vl2  (3 x float4)
//   FP32  32 B: x0 x1 x2 v0 | v1 v2 - -                             (2 x float4)
#pragma once

#include "engine.h"

namespace tg {
namespace {

template <int PREC>
struct St {
    float x[3], v[3], xl[3], vl[3];
};
template <>
struct St<P_FP64> {
    double x[3], v[3], xl[3], vl[3];
};

template <int PREC>
__device__ __forceinline__ St<PREC> load_state(const void *buf, int64_t g) {
    St<PREC> s;
    if constexpr (PREC == P_FP64) {
        const double2 *p = reinterpret_cast<const double2 *>(buf) + 3 * g;
        double2 a0 = __ldg(p), a1 = __ldg(p + 1), a2 = __ldg(p + 2);
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a1.x;
        s.v[0] = a1.y; s.v[1] = a2.x; s.v[2] = a2.y;
    } else if constexpr (PREC == P_FP32C) {
        const float4 *p = reinterpret_cast<const float4 *>(buf) + 3 * g;
        float4 a0 = __ldg(p), a1 = __ldg(p + 1), a2 = __ldg(p + 2);
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a0.z;
        s.v[0] = a0.w; s.v[1] = a1.x; s.v[2] = a1.y;
        s.xl[0] = a1.z; s.xl[1] = a1.w; s.xl[2] = a2.x;
        s.vl[0] = a2.y; s.vl[1] = a2.z; s.vl[2] = a2.w;
    } else {
        const float4 *p = reinterpret_cast<const float4 *>(buf) + 2 * g;
        float4 a0 = __ldg(p);
        float2 a1 = __ldg(reinterpret_cast<const float2 *>(p + 1));
        s.x[0] = a0.x; s.x[1] = a0.y; s.x[2] = a0.z;
        s.v[0] = a0.w; s.v[1] = a1.x; s.v[2] = a1.y;
        s.xl[0] = s.xl[1] = s.xl[2] = 0.f;  // the epilogue adds the (zero) low parts
        s.vl[0] = s.vl[1] = s.vl[2] = 0.f;
    }
    return s;
}

template <int PREC>
__device__ __forceinline__ void store_state(void *buf, int64_t g, const St<PREC> &s) {
    if constexpr (PREC == P_FP64) {
        double2 *p = reinterpret_cast<double2 *>(buf) + 3 * g;
        p[0] = make_double2(s.x[0], s.x[1]);
        p[1] = make_double2(s.x[2], s.v[0]);
        p[2] = make_double2(s.v[1], s.v[2]);
    } else if constexpr (PREC == P_FP32C) {
        float4 *p = reinterpret_cast<float4 *>(buf) + 3 * g;
        p[0] = make_float4(s.x[0], s.x[1], s.x[2], s.v[0]);
        p[1] = make_float4(s.v[1], s.v[2], s.xl[0], s.xl[1]);
        p[2] = make_float4(s.xl[2], s.vl[0], s.vl[1], s.vl[2]);
    } else {
        float4 *p = reinterpret_cast<float4 *>(buf) + 2 * g;
        p[0] = make_float4(s.x[0], s.x[1], s.x[2], s.v[0]);
        p[1] = make_float4(s.v[1], s.v[2], 0.f, 0.f);
    }
}

}  // namespace
}  // namespace tg
