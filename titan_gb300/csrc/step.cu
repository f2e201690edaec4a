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
//
// State records (one per mass, tiled order), loaded with 16-byte vectors:
//   FP64  48 B: x0 x1 | x2 v0 | v1 v2                (3 x double2)
//   FP32C 48 B: xh0 xh1 xh2 vh0 | vh1 vh2 xl0 xl1 | xl2 vl0 vl1 vl2  (3 x float4)
//   FP32  32 B: x0 x1 x2 v0 | v1 v2 - -              (2 x float4)
#include <cstdint>

#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"

namespace tg {

namespace {

constexpr int kBatchB = 4;     // slab entries in flight per thread (phase B)
constexpr int kBatchC = 4;     // 8-byte incidence words in flight per thread (phase C)
constexpr int kPrefetchW = 8;  // incidence words (32 codes) fetched before phase B

// ------------------------------------------------------------- kernel -----
template <int PREC>
__global__ void __launch_bounds__(512) k_step(StepArgs a, int parity, int write_acc) {
    using R = typename Real<PREC>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const TileInfo ti = a.tiles[blockIdx.x];
    const int S = ti.nm + ti.nh, E = ti.ne;
    R *sx = reinterpret_cast<R *>(smem_raw);  // 3*S positions (hi)
    R *sv = sx + 3 * S;                        // 3*S velocities (hi)
    R *sxl = sv + 3 * S;                       // 3*S position lo (FP32C only)
    R *sF = (PREC == P_FP32C) ? sxl + 3 * S : sxl;  // 3*E entry forces
    R *sH = sF + 3 * E;                        // 3*nheavy heavy-mass sums
    const void *in = parity ? a.state1 : a.state0;
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const double T = a.tbuf[parity];
    if (blockIdx.x == 0 && threadIdx.x == 0) a.tbuf[parity ^ 1] = T + prm->dt;

    // per-mass inputs of phase C for this thread's own mass, issued now so
    // that their latency hides behind phases A and B
    const int i_own = threadIdx.x;
    uint8_t fl_own = MF_FIXED;
    uint32_t d_own = 0, woff_own = 0;
    R m_own = 1;
    float vl_own[3] = {0.f, 0.f, 0.f};
    uint2 cw_own[kPrefetchW];
    if (i_own < ti.nm) {
        const int64_t g = (int64_t)ti.mass_off + i_own;
        fl_own = __ldg(a.flags + g);
        d_own = __ldg(a.deg + g);
        m_own = __ldg(reinterpret_cast<const R *>(a.mass) + g);
        woff_own = __ldg(a.warp_inc_off + ti.warp_off + (i_own >> 5));
        if constexpr (PREC == P_FP32C) {
            const float4 a2 = __ldg(reinterpret_cast<const float4 *>(in) + 3 * g + 2);
            vl_own[0] = a2.y;
            vl_own[1] = a2.z;
            vl_own[2] = a2.w;
        }
    }

    // ---- A: stage tile + halo (two records in flight per thread) ---------
    for (int i0 = threadIdx.x; i0 < S; i0 += 2 * blockDim.x) {
        const int i1 = i0 + blockDim.x;
        const int64_t g0 = i0 < ti.nm ? (int64_t)ti.mass_off + i0 : (int64_t)__ldg(a.halo + ti.halo_off + i0 - ti.nm);
        int64_t g1 = g0;
        if (i1 < S) g1 = i1 < ti.nm ? (int64_t)ti.mass_off + i1 : (int64_t)__ldg(a.halo + ti.halo_off + i1 - ti.nm);
        const St<PREC> s0 = load_state<PREC>(in, g0);
        St<PREC> s1 = s0;
        if (i1 < S) s1 = load_state<PREC>(in, g1);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            sx[c * S + i0] = s0.x[c];
            sv[c * S + i0] = s0.v[c];
            if constexpr (PREC == P_FP32C) sxl[c * S + i0] = s0.xl[c];
            if (i1 < S) {
                sx[c * S + i1] = s1.x[c];
                sv[c * S + i1] = s1.v[c];
                if constexpr (PREC == P_FP32C) sxl[c * S + i1] = s1.xl[c];
            }
        }
    }
    // the first incidence words of this thread's mass (needs woff_own, d_own)
    if (i_own < ti.nm && d_own != 255) {
        const uint2 *ip = reinterpret_cast<const uint2 *>(a.inc + woff_own) + (i_own & 31);
        const uint32_t nw = (d_own + 3) >> 2;
#pragma unroll
        for (int w = 0; w < kPrefetchW; w++)
            if ((uint32_t)w < nw) cw_own[w] = __ldg(ip + 32 * w);
    }
    __syncthreads();

    // ---- B: one force per slab entry --------------------------------------
    if constexpr (PREC == P_FP64) {
        const double *ent = reinterpret_cast<const double *>(a.ent) + 4 * (int64_t)ti.ent_off;
        const double *act = reinterpret_cast<const double *>(a.act) + 4 * (int64_t)ti.ent_off;
        for (int e0 = threadIdx.x; e0 < E; e0 += kBatchB * blockDim.x) {
            D4 r[kBatchB], q[kBatchB];
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                int e = e0 + k * blockDim.x;
                if (e < E) r[k] = ldg_d4(ent + 4 * e);
                if (e < ti.nact) q[k] = ldg_d4(act + 4 * e);
            }
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                int e = e0 + k * blockDim.x;
                if (e >= E) break;
                uint32_t ends = (uint32_t)__double_as_longlong(r[k].w);
                int sa = ends & 0xfff, sb = (ends >> 12) & 0xfff;
                double scale = 1.0;
                if (e < ti.nact) {
                    double th = q[k].x * T;
                    th = th + q[k].z;
                    double s = q[k].y * sin(th);
                    scale = ((ends >> 24) & 3) == 2 ? 1.0 - s : 1.0 + s;
                }
                double d0 = sx[sb] - sx[sa], d1 = sx[S + sb] - sx[S + sa], d2 = sx[2 * S + sb] - sx[2 * S + sa];
                double nrm = nrm3(d0, d1, d2);
                double u0 = d0 / nrm, u1 = d1 / nrm, u2 = d2 / nrm;
                double fs = r[k].x * (r[k].y * scale - nrm);
                double f0 = u0 * fs, f1 = u1 * fs, f2 = u2 * fs;
                if (r[k].z != 0.0) {
                    double w0 = sv[sa] - sv[sb], w1 = sv[S + sa] - sv[S + sb], w2 = sv[2 * S + sa] - sv[2 * S + sb];
                    double dd = ((w0 * u0 + w1 * u1) + w2 * u2) * r[k].z;
                    f0 = f0 + u0 * dd;
                    f1 = f1 + u1 * dd;
                    f2 = f2 + u2 * dd;
                }
                sF[e] = f0;
                sF[E + e] = f1;
                sF[2 * E + e] = f2;
            }
        }
    } else {
        const float4 *ent = reinterpret_cast<const float4 *>(a.ent) + ti.ent_off;
        const float4 *act = reinterpret_cast<const float4 *>(a.act) + ti.ent_off;
        const float Thi = (float)T;
        const float Tlo = (float)(T - (double)Thi);
        for (int e0 = threadIdx.x; e0 < E; e0 += kBatchB * blockDim.x) {
            float4 r[kBatchB], q[kBatchB];
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                int e = e0 + k * blockDim.x;
                if (e < E) r[k] = __ldg(ent + e);
                if (e < ti.nact) q[k] = __ldg(act + e);
            }
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                int e = e0 + k * blockDim.x;
                if (e >= E) break;
                uint32_t ends = __float_as_uint(r[k].x);
                int sa = ends & 0xfff, sb = (ends >> 12) & 0xfff;
                float rs = r[k].z;
                if (e < ti.nact) {
                    float th = fmaf(q[k].x, Thi, fmaf(q[k].x, Tlo, q[k].z));
                    float s = q[k].y * sinf(th);
                    rs = r[k].z * (((ends >> 24) & 3) == 2 ? 1.0f - s : 1.0f + s);
                }
                float d0 = sx[sb] - sx[sa], d1 = sx[S + sb] - sx[S + sa], d2 = sx[2 * S + sb] - sx[2 * S + sa];
                if constexpr (PREC == P_FP32C) {
                    d0 += sxl[sb] - sxl[sa];
                    d1 += sxl[S + sb] - sxl[S + sa];
                    d2 += sxl[2 * S + sb] - sxl[2 * S + sa];
                }
                float nrm = nrm3f(d0, d1, d2);
                float inv = __frcp_rn(nrm);
                float u0 = d0 * inv, u1 = d1 * inv, u2 = d2 * inv;
                float f = r[k].y * (rs - nrm);
                if (r[k].w != 0.f) {
                    float w0 = sv[sa] - sv[sb], w1 = sv[S + sa] - sv[S + sb], w2 = sv[2 * S + sa] - sv[2 * S + sb];
                    f = fmaf(fmaf(w2, u2, fmaf(w1, u1, w0 * u0)), r[k].w, f);
                }
                sF[e] = u0 * f;
                sF[E + e] = u1 * f;
                sF[2 * E + e] = u2 * f;
            }
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
                sH[ti.nheavy + h] = p1;
                sH[2 * ti.nheavy + h] = p2;
            }
        }
        __syncthreads();
    }

    // ---- C: per-mass gather, constraints, integration ----------------------
    for (int i = threadIdx.x; i < ti.nm; i += blockDim.x) {
        const int64_t g = (int64_t)ti.mass_off + i;
        const bool own = i == i_own;
        const uint8_t fl = own ? fl_own : __ldg(a.flags + g);
        if (fl & MF_FIXED) continue;  // src/sim.cu:1100
        const uint32_t d = own ? d_own : __ldg(a.deg + g);
        const R m = own ? m_own : __ldg(reinterpret_cast<const R *>(a.mass) + g);
        R F0 = 0, F1 = 0, F2 = 0;
        // codes 4w..4w+3 of one incidence word, in ascending order
        auto add_word = [&](const uint2 cw, uint32_t w) {
#pragma unroll
            for (int h = 0; h < 4; h++) {
                const uint32_t j = 4 * w + h;
                if (j < d) {
                    const uint32_t word = h < 2 ? cw.x : cw.y;
                    const uint32_t code = (word >> (16 * (h & 1))) & 0xffffu;
                    const int idx = code & 0x7fff;
                    if (code & 0x8000) {
                        F0 = F0 + (-sF[idx]);
                        F1 = F1 + (-sF[E + idx]);
                        F2 = F2 + (-sF[2 * E + idx]);
                    } else {
                        F0 = F0 + sF[idx];
                        F1 = F1 + sF[E + idx];
                        F2 = F2 + sF[2 * E + idx];
                    }
                }
            }
        };
        if (d == 255) {
            int h = 0;
            while (h < ti.nheavy && a.heavy_local[ti.heavy_off + h] != i) h++;
            F0 = F0 + sH[h];
            F1 = F1 + sH[ti.nheavy + h];
            F2 = F2 + sH[2 * ti.nheavy + h];
        } else if (d > 0) {
            const uint32_t woff = own ? woff_own : __ldg(a.warp_inc_off + ti.warp_off + (i >> 5));
            const uint2 *ip = reinterpret_cast<const uint2 *>(a.inc + woff) + (i & 31);
            const uint32_t nw = (d + 3) >> 2;
            uint32_t w0 = 0;
            if (own) {
#pragma unroll
                for (int w = 0; w < kPrefetchW; w++)
                    if ((uint32_t)w < nw) add_word(cw_own[w], w);
                w0 = kPrefetchW;
            }
            for (; w0 < nw; w0 += kBatchC) {
                uint2 cw[kBatchC];
#pragma unroll
                for (int k = 0; k < kBatchC; k++)
                    if (w0 + k < nw) cw[k] = __ldg(ip + 32 * (w0 + k));
#pragma unroll
                for (int k = 0; k < kBatchC; k++)
                    if (w0 + k < nw) add_word(cw[k], w0 + k);
            }
        }
        St<PREC> s;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            s.x[c] = sx[c * S + i];
            s.v[c] = sv[c * S + i];
        }
        if constexpr (PREC == P_FP32C) {
#pragma unroll
            for (int c = 0; c < 3; c++) s.xl[c] = sxl[c * S + i];
            if (own) {
                s.vl[0] = vl_own[0];
                s.vl[1] = vl_own[1];
                s.vl[2] = vl_own[2];
            } else {
                const float4 a2 = __ldg(reinterpret_cast<const float4 *>(in) + 3 * g + 2);
                s.vl[0] = a2.y;
                s.vl[1] = a2.z;
                s.vl[2] = a2.w;
            }
        } else if constexpr (PREC == P_FP32) {
#pragma unroll
            for (int c = 0; c < 3; c++) s.xl[c] = s.vl[c] = 0.f;
        }
        integrate<PREC>(a, ti, g, fl, m, F0, F1, F2, s, out, write_acc, np, prm);
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
    const St<PREC> s = load_state<PREC>(a.parity ? a.state1 : a.state0, g);
    const int64_t np = a.npad;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double x = (double)s.x[c], v = (double)s.v[c];
        if constexpr (PREC == P_FP32C) {
            x += (double)s.xl[c];
            v += (double)s.vl[c];
        }
        if (a.pos) a.pos[3 * i + c] = x;
        if (a.vel) a.vel[3 * i + c] = v;
        if (a.accout) a.accout[3 * i + c] = (double)reinterpret_cast<const R *>(a.acc)[c * np + g];
    }
}

// Writes pos and/or vel of the listed masses into both buffers, keeping the
// other field from the current buffer.
template <int PREC>
__global__ void k_scatter(XferArgs a) {
    using R = typename Real<PREC>::T;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    int64_t src = a.idx ? a.idx[i] : i;
    int64_t g = a.old2new[src];
    const int64_t np = a.npad;
    St<PREC> s = load_state<PREC>(a.parity ? a.state1 : a.state0, g);
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (a.ipos) {
            double x = a.ipos[3 * i + c];
            s.x[c] = (R)x;
            if constexpr (PREC == P_FP32C) s.xl[c] = (R)(x - (double)s.x[c]);
        }
        if (a.ivel) {
            double v = a.ivel[3 * i + c];
            s.v[c] = (R)v;
            if constexpr (PREC == P_FP32C) s.vl[c] = (R)(v - (double)s.v[c]);
        }
        if (a.ipos) reinterpret_cast<R *>(a.acc)[c * np + g] = (R)0;
    }
    store_state<PREC>(a.state0, g, s);
    store_state<PREC>(a.state1, g, s);
}

// ------------------------------------------------------ diagnostics -------
// Pass 1: each of kDiagBlocks blocks sums a fixed grid-stride share in FP64
// and reduces it with a fixed tree; pass 2 reduces the partials the same way.
template <int PREC>
__global__ void __launch_bounds__(256) k_diag1(DiagArgs a) {
    __shared__ double red[kDiagQ][256];
    double q[kDiagQ];
#pragma unroll
    for (int k = 0; k < kDiagQ; k++) q[k] = 0.0;
    using R = typename Real<PREC>::T;
    const R *ms = reinterpret_cast<const R *>(a.mass);
    auto pos = [&](const St<PREC> &s, int c) {
        double x = (double)s.x[c];
        if constexpr (PREC == P_FP32C) x += (double)s.xl[c];
        return x;
    };
    auto vel = [&](const St<PREC> &s, int c) {
        double v = (double)s.v[c];
        if constexpr (PREC == P_FP32C) v += (double)s.vl[c];
        return v;
    };
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < a.n; g += stride) {
        const St<PREC> s = load_state<PREC>(a.state, g);
        double m = (double)ms[g];
        double x[3] = {pos(s, 0), pos(s, 1), pos(s, 2)};
        double v[3] = {vel(s, 0), vel(s, 1), vel(s, 2)};
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
        const St<PREC> sl = load_state<PREC>(a.state, l), sr = load_state<PREC>(a.state, r);
        double d0 = pos(sl, 0) - pos(sr, 0), d1 = pos(sl, 1) - pos(sr, 1), d2 = pos(sl, 2) - pos(sr, 2);
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

int state_words(int precision) { return precision == P_FP64 ? 6 : (precision == P_FP32C ? 12 : 8); }

size_t tile_smem_bytes(int precision, int slots, int entries, int heavy) {
    size_t words = (size_t)(precision == P_FP32C ? 9 : 6) * slots + 3 * (size_t)entries + 3 * (size_t)heavy;
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
