// step_async.cu -- per-tile step kernel with asynchronous staging (sm_103a).
//
// Same tiles, arithmetic, summation order and results as k_step
// (step_kernel.cuh) -- the tests check them bit for bit -- but every global
// read of phases A and B is issued at once, before the CTA waits:
//   * one thread starts two bulk copies on the Tensor Memory Accelerator
//     (cp.async.bulk with an mbarrier transaction count): the tile's slab
//     records straight into the force slots, and the tile masses' state
//     records;
//   * all threads gather the halo state records with 16-byte cp.async and
//     load the actuation records of their first entries into registers;
//   * then one bounded wait, and phase B computes each entry's force from
//     the record in its slot and writes the force over it (each slot is read
//     and written by the same thread).
// The per-tile kernel instead reads slab records in small register batches,
// each a separate round trip to memory.  Shared memory is the same plus the
// mbarrier.  A wait that times out sets *err, drains (bounded) and returns.
#include <cstdint>

#include "async_copy.cuh"
#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

constexpr int kActPf = 4;   // actuation records per thread fetched before the wait
constexpr int kBatchC = 4;  // incidence words in flight per thread (phase C)

__host__ __device__ constexpr int64_t al16(int64_t x) { return (x + 15) & ~int64_t(15); }

template <int PREC>
__host__ __device__ constexpr int rec_b() { return PREC == P_FP32 ? 32 : 48; }

template <int PREC>
__global__ void __launch_bounds__(512) k_step_async(StepArgs a, int parity, int write_acc) {
    using R = typename Real<PREC>::T;
    constexpr int kRec = rec_b<PREC>();
    constexpr int kSlot = Slot<PREC>::kBytes;
    constexpr int kChunks = kRec / 16;
    extern __shared__ __align__(128) uint8_t smem[];
    const TileInfo ti = a.tiles[blockIdx.x];
    const int S = ti.nm + ti.nh, E = ti.ne;
    uint8_t *st = smem;
    uint8_t *slots = smem + al16((int64_t)S * kRec);
    R *sH = reinterpret_cast<R *>(slots + (int64_t)(E + 1) * kSlot);  // after the zero slot
    uint64_t *bar = reinterpret_cast<uint64_t *>(
        smem + al16(al16((int64_t)S * kRec) + (int64_t)(E + 1) * kSlot + 3 * (int64_t)ti.nheavy * (int64_t)sizeof(R)));
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const StepTime t = step_time(a.tbuf[parity]);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.tbuf[parity ^ 1] = t.T + prm->launch_dt;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint8_t *ent = reinterpret_cast<const uint8_t *>(a.ent) + (int64_t)ti.ent_off * kSlot;
    const uint8_t *act = reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * kSlot;
    if (threadIdx.x == 0) {
        fence_proxy_async();
        const uint32_t eb = (uint32_t)E * kSlot, sb = (uint32_t)ti.nm * kRec;
        mbar_expect_tx(bar, eb + sb);
        issue_chunks(slots, ent, eb, bar);
        issue_chunks(st, in + (int64_t)ti.mass_off * kRec, sb, bar);
    }
    // halo records, 16 bytes per copy
    for (int q = threadIdx.x; q < ti.nh * kChunks; q += blockDim.x) {
        const int h = q / kChunks, c = q - h * kChunks;
        const int64_t g = __ldg(a.halo + ti.halo_off + h);
        cp_async16(st + (int64_t)(ti.nm + h) * kRec + 16 * c, in + g * kRec + 16 * c);
    }
    cp_async_commit();

    // phase-C inputs of this thread's own mass and its first actuation
    // records, in flight while the copies land
    const int i_own = threadIdx.x;
    uint8_t fl_own = MF_FIXED;
    uint32_t d_own = 0, woff_own = 0;
    R m_own = 1;
    if (i_own < ti.nm) {
        const int64_t g = (int64_t)ti.mass_off + i_own;
        fl_own = __ldg(a.flags + g);
        d_own = __ldg(a.deg + g);
        m_own = __ldg(reinterpret_cast<const R *>(a.mass) + g);
        woff_own = __ldg(a.warp_inc_off + ti.warp_off + (i_own >> 5));
    }
    Rec16<PREC> qa[kActPf];
#pragma unroll
    for (int k = 0; k < kActPf; k++) {
        const int e = threadIdx.x + k * blockDim.x;
        if (e < ti.nact) qa[k] = ldcs_rec<PREC>(act + (int64_t)e * kSlot);
    }

    cp_async_wait_all();
    bool landed = false;
    for (uint32_t it = 0; it < kWaitLimit && !landed; it++) landed = mbar_try_wait(bar, 0);
    if (__syncthreads_or(!landed)) {  // block-uniform
        if (threadIdx.x == 0) atomicOr(a.err, 1);
        for (uint32_t it = 0; it < kWaitLimit && !mbar_try_wait(bar, 0); it++) {
        }
        return;
    }

    // ---- B: one force per slab entry, written over its record ------------
    {
        Rec16<PREC> r[kActPf];
#pragma unroll
        for (int k = 0; k < kActPf; k++) {
            const int e = threadIdx.x + k * blockDim.x;
            if (e < E) r[k] = load_rec<PREC>(slots + (int64_t)e * kSlot);
        }
#pragma unroll
        for (int k = 0; k < kActPf; k++) {
            const int e = threadIdx.x + k * blockDim.x;
            if (e < E) entry_force<PREC>(r[k], e < ti.nact, qa[k], st, t, slots + (int64_t)e * kSlot);
        }
        for (int e = threadIdx.x + kActPf * blockDim.x; e < E; e += blockDim.x) {
            const Rec16<PREC> rr = load_rec<PREC>(slots + (int64_t)e * kSlot);
            const bool actuated = e < ti.nact;
            const Rec16<PREC> qq = actuated ? ldcs_rec<PREC>(act + (int64_t)e * kSlot) : rr;
            entry_force<PREC>(rr, actuated, qq, st, t, slots + (int64_t)e * kSlot);
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
            for (uint32_t w0 = 0; w0 < nw; w0 += kBatchC) {
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
        integrate<PREC>(a, ti, g, fl, m, F0, F1, F2, s, out, g, write_acc, np, prm);
    }
}

}  // namespace

size_t tile_async_smem_bytes(int precision, int slots, int entries, int heavy) {
    return (size_t)al16((int64_t)tile_smem_bytes(precision, slots, entries, heavy)) + 16;
}

cudaError_t step_async_prepare(int precision, size_t smem) {
    const void *f = precision == P_FP64   ? (const void *)k_step_async<P_FP64>
                    : precision == P_FP32 ? (const void *)k_step_async<P_FP32>
                                          : (const void *)k_step_async<P_FP32C>;
    return raise_smem_limit(f, smem);
}

cudaError_t launch_step_async(int precision, const StepArgs &a, int ntiles, int threads, size_t smem, int parity,
                              int write_acc, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    switch (precision) {
        case P_FP64: k_step_async<P_FP64><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
        case P_FP32: k_step_async<P_FP32><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
        default: k_step_async<P_FP32C><<<ntiles, threads, smem, s>>>(a, parity, write_acc); break;
    }
    return cudaGetLastError();
}

}  // namespace tg
