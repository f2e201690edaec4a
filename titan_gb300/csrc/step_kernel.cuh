// step_kernel.cuh -- the per-tile step kernel (one CTA per tile), shared by
// the translation units that instantiate its launch-bound variants.
//
// One CTA per tile (plan.h).  Per step and tile:
//   A. stage the state records of the tile's masses and of its halo in
//      shared memory (16-byte vector copies, two records in flight per
//      thread);
//   B. compute every slab entry's spring force once (src/sim.cu:1054-1065)
//      into its shared-memory force slot (tile_phases.cuh);
//   C. per mass, sum its incident slots in ascending spring order (one legal
//      serialisation of the reference's atomics, src/vec.cu:33-37), then
//      the per-mass epilogue (epilogue.cuh: src/sim.cu:1100-1166) writes the
//      other ping-pong buffer.
// A thread's own mass's phase-C inputs (flags, degree, m, incidence words)
// are fetched before phase A so that their latency hides behind A and B.
// Kernels are compiled without FMA contraction (build flag --fmad=false):
// the FP64 form then rounds each operation as the CPU oracle does.
//
// LBT / LBM are the kernel's launch bounds (threads per CTA, minimum CTAs
// per SM): they cap registers per thread at 65536 / (LBT * LBM), trading
// registers for resident warps.  INTEG is the integrator (INTEG_*), fixed at
// compile time so that each instance carries only its own update.
#pragma once

#include <cstdint>

#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

constexpr int kBatchC = 4;  // 8-byte incidence words in flight per thread (phase C)

// incidence words (4 codes each) of a thread's own mass fetched before
// phase B; none under a register cap
template <int LBM>
__host__ __device__ constexpr int prefetch_w() { return LBM >= 3 ? 0 : 7; }

// slab entries in flight per thread in phase B (FP64 records are 32 B)
template <int PREC, int LBM>
__host__ __device__ constexpr int batch_b() { return (PREC == P_FP64 || LBM >= 3) ? 2 : 4; }

template <int PREC>
__host__ __device__ constexpr int rec_bytes() { return PREC == P_FP32 ? 32 : 48; }

__host__ __device__ constexpr int64_t align16(int64_t x) { return (x + 15) & ~int64_t(15); }

template <int PREC>
__device__ __forceinline__ void copy_record(uint8_t *dst, const uint8_t *src) {
    constexpr int kV = rec_bytes<PREC>() / 16;
#pragma unroll
    for (int v = 0; v < kV; v++)
        reinterpret_cast<float4 *>(dst)[v] = __ldg(reinterpret_cast<const float4 *>(src) + v);
}

// One step of one tile by the whole CTA (phases A, B, C above) in the
// dynamic shared memory smem (tile_smem_bytes).  first_tile: this CTA
// advances the scene's time record.  Callers synchronise the CTA before
// reusing smem.  L2ONLY: the state and time records are read around L1 (a
// persistent kernel in which other CTAs wrote them since this SM may have
// cached them); a kernel launched per step reads them through L1.
template <int PREC, int LBM, int INTEG, bool L2ONLY = false>
__device__ __forceinline__ void tile_step(const StepArgs &a, const TileInfo &ti, uint8_t *smem, int parity,
                                          int write_acc, bool first_tile) {
    using R = typename Real<PREC>::T;
    constexpr int kRec = rec_bytes<PREC>();
    constexpr int kSlot = Slot<PREC>::kBytes;
    const int S = ti.nm + ti.nh, E = ti.ne;
    uint8_t *st = smem;                                   // S state records
    uint8_t *slots = smem + align16((int64_t)S * kRec);   // E force slots
    R *sH = reinterpret_cast<R *>(slots + (int64_t)(E + 1) * kSlot);  // 3 * nheavy, after the zero slot
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const StepTime t = step_time(L2ONLY ? __ldcg(a.tbuf + parity) : a.tbuf[parity]);
    if (first_tile && threadIdx.x == 0) a.tbuf[parity ^ 1] = t.T + prm->launch_dt;

    // phase-C inputs of this thread's own mass, issued first
    const int i_own = threadIdx.x;
    uint8_t fl_own = MF_FIXED;
    uint32_t d_own = 0, woff_own = 0;
    R m_own = 1;
    constexpr int kPrefetchW = prefetch_w<LBM>();
    uint2 cw_own[kPrefetchW > 0 ? kPrefetchW : 1];
    if (i_own < ti.nm) {
        const int64_t g = (int64_t)ti.mass_off + i_own;
        fl_own = __ldg(a.flags + g);
        d_own = __ldg(a.deg + g);
        m_own = __ldg(reinterpret_cast<const R *>(a.mass) + g);
        woff_own = __ldg(a.warp_inc_off + ti.warp_off + (i_own >> 5));
    }

    // ---- A: stage tile + halo records, two in flight per thread ---------
    for (int i0 = threadIdx.x; i0 < S; i0 += 2 * blockDim.x) {
        const int i1 = i0 + blockDim.x;
        const int64_t g0 = i0 < ti.nm ? (int64_t)ti.mass_off + i0 : (int64_t)__ldg(a.halo + ti.halo_off + i0 - ti.nm);
        int64_t g1 = g0;
        if (i1 < S) g1 = i1 < ti.nm ? (int64_t)ti.mass_off + i1 : (int64_t)__ldg(a.halo + ti.halo_off + i1 - ti.nm);
        float4 v0[kRec / 16], v1[kRec / 16];
#pragma unroll
        for (int v = 0; v < kRec / 16; v++) {
            const float4 *p = reinterpret_cast<const float4 *>(in + g0 * kRec) + v;
            v0[v] = L2ONLY ? __ldcg(p) : __ldg(p);
        }
        if (i1 < S) {
#pragma unroll
            for (int v = 0; v < kRec / 16; v++) {
                const float4 *p = reinterpret_cast<const float4 *>(in + g1 * kRec) + v;
                v1[v] = L2ONLY ? __ldcg(p) : __ldg(p);
            }
        }
#pragma unroll
        for (int v = 0; v < kRec / 16; v++) reinterpret_cast<float4 *>(st + (int64_t)i0 * kRec)[v] = v0[v];
        if (i1 < S) {
#pragma unroll
            for (int v = 0; v < kRec / 16; v++) reinterpret_cast<float4 *>(st + (int64_t)i1 * kRec)[v] = v1[v];
        }
    }
    // the first incidence words of this thread's mass
    if (i_own < ti.nm && d_own != 255) {
        const uint2 *ip = reinterpret_cast<const uint2 *>(a.inc + woff_own) + (i_own & 31);
        const uint32_t nw = (d_own + 3) >> 2;
#pragma unroll
        for (int w = 0; w < kPrefetchW; w++)
            if ((uint32_t)w < nw) cw_own[w] = __ldcs(ip + 32 * w);
    }
    __syncthreads();

    // ---- B: one force per slab entry (kBatchB records in flight) ----------
    {
        const uint8_t *ent = reinterpret_cast<const uint8_t *>(a.ent) + (int64_t)ti.ent_off * kSlot;
        const uint8_t *act = reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * kSlot;
        constexpr int kBatchB = batch_b<PREC, LBM>();
        for (int e0 = threadIdx.x; e0 < E; e0 += kBatchB * blockDim.x) {
            Rec16<PREC> r[kBatchB], q[kBatchB];
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                const int e = e0 + k * blockDim.x;
                if (e < E) r[k] = ldcs_rec<PREC>(ent + (int64_t)e * kSlot);
                if (e < ti.nact) q[k] = ldcs_rec<PREC>(act + (int64_t)e * kSlot);
            }
#pragma unroll
            for (int k = 0; k < kBatchB; k++) {
                const int e = e0 + k * blockDim.x;
                if (e >= E) break;
                entry_force<PREC>(r[k], e < ti.nact, q[k], st, t, slots + (int64_t)e * kSlot);
            }
        }
    }
    // the zero force that padding incidence codes name (slot E)
    if (threadIdx.x == 0) {
        reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[0] = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (kSlot == 32)
            reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[1] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();

    // ---- C0: heavy masses --------------------------------------------------
    if (ti.nheavy > 0) {
        heavy_sums<PREC>(a, ti, slots, sH, threadIdx.x >> 5, blockDim.x >> 5);
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
                    if ((uint32_t)w < nw) gather_word_padded<PREC>(slots, cw_own[w], F0, F1, F2);
                w0 = kPrefetchW;
            }
            for (; w0 < nw; w0 += kBatchC) {
                uint2 cw[kBatchC];
#pragma unroll
                for (int k = 0; k < kBatchC; k++)
                    if (w0 + k < nw) cw[k] = __ldcs(ip + 32 * (w0 + k));
#pragma unroll
                for (int k = 0; k < kBatchC; k++)
                    if (w0 + k < nw) gather_word_padded<PREC>(slots, cw[k], F0, F1, F2);
            }
        }
        St<PREC> s = load_state_smem<PREC>(st, i);
        integrate<PREC, INTEG>(a, ti, g, fl, m, F0, F1, F2, s, out, g, write_acc, np, prm);
    }
}

template <int PREC, int LBT, int LBM, int INTEG>
__global__ void __launch_bounds__(LBT, LBM) k_step(StepArgs a, int parity, int write_acc) {
    extern __shared__ __align__(16) uint8_t smem[];
    const TileInfo ti = a.tiles[blockIdx.x];
    tile_step<PREC, LBM, INTEG>(a, ti, smem, parity, write_acc, blockIdx.x == 0);
}

}  // namespace

}  // namespace tg
