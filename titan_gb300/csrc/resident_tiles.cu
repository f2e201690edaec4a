// resident_tiles.cu -- self-contained tiles, all steps in one launch.
//
// A tile with no halo (every spring of its masses has both ends in the
// tile) needs nothing from other tiles between steps.  One CTA takes such a
// tile, stages its masses' state records in shared memory twice (current
// and next state) -- and, when they fit, its slab, actuation and incidence
// records once per launch -- and runs every requested step there with the
// per-step kernel's phases:
//   B. every slab entry's spring force once into its force slot
//      (entry_force, src/sim.cu:1054-1065);
//   C. per mass, the sum of its incident slots in ascending spring order
//      (gather_word_padded; heavy masses by heavy_sums), then the per-mass
//      epilogue (integrate, src/sim.cu:1100-1166) into the other buffer.
// Two barriers per step, no global-memory traffic for the state until the
// last step, whose records (and accelerations) go to the output buffer.
// The functions and the order of every sum are the per-step kernels': the
// results are bit-identical to them, and in FP64 to the CPU oracle.
//
// Symplectic Euler only (the host keeps the other integrators on the
// per-step kernels).  The launch parameters are copied to shared memory
// once per CTA.  The time of the first step comes from its own record, so
// that per-step kernels advancing the time record may run concurrently (on
// another stream: their masses and the resident tiles' are disjoint).
#include <cstdint>

#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

template <int PREC>
__host__ __device__ constexpr int rt_rec_bytes() { return PREC == P_FP32 ? 32 : 48; }

__host__ __device__ constexpr int64_t rt_align16(int64_t x) { return (x + 15) & ~int64_t(15); }

constexpr int64_t kParamBytes = (int64_t)sizeof(DevParams);  // a multiple of 16

// Byte offsets of one tile's shared-memory regions.
struct RtLayout {
    int64_t st0, st1, slots, heavy, ent, act, inc, total;
};

__host__ __device__ inline RtLayout rt_layout(int precision, const TileInfo &ti, int stage) {
    const int64_t rec = precision == P_FP32 ? 32 : 48;
    const int64_t slot = precision == P_FP64 ? 32 : 16;
    const int64_t rs = precision == P_FP64 ? 8 : 4;
    RtLayout L;
    L.st0 = kParamBytes;
    L.st1 = L.st0 + rt_align16((int64_t)ti.nm * rec);
    L.slots = L.st1 + rt_align16((int64_t)ti.nm * rec);
    L.heavy = L.slots + ((int64_t)ti.ne + 1) * slot;  // + the zero slot padding codes name
    L.ent = L.heavy + rt_align16(3 * (int64_t)ti.nheavy * rs);
    L.act = L.ent + (stage ? (int64_t)ti.ne * slot : 0);
    L.inc = L.act + (stage ? (int64_t)ti.nact * slot : 0);
    L.total = L.inc + (stage ? rt_align16((int64_t)ti.inc_words * 2) : 0);
    return L;
}

template <int PREC, int MPT, int STAGE>
__global__ void __launch_bounds__(512) k_tile_resident(StepArgs a, TileResArgs r, int parity, int64_t nsteps,
                                                       int write_acc) {
    using R = typename Real<PREC>::T;
    constexpr int kRec = rt_rec_bytes<PREC>();
    constexpr int kSlot = Slot<PREC>::kBytes;
    extern __shared__ __align__(16) uint8_t smem[];
    const DevParams *prm = reinterpret_cast<const DevParams *>(smem);
    for (int v = threadIdx.x; v < (int)(kParamBytes / 16); v += blockDim.x)
        reinterpret_cast<float4 *>(smem)[v] = __ldg(reinterpret_cast<const float4 *>(a.prm) + v);
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    uint8_t *out = reinterpret_cast<uint8_t *>((parity ^ (int)(nsteps & 1)) ? a.state1 : a.state0);
    const int64_t np = a.npad;
    const double T0 = *r.t0;
    const int nwarps = blockDim.x >> 5;

    for (int t = blockIdx.x; t < r.ntiles; t += gridDim.x) {
        const TileInfo ti = r.tiles[t];
        const int nm = ti.nm, E = ti.ne;
        const RtLayout L = rt_layout(PREC, ti, STAGE);
        uint8_t *const st0 = smem + L.st0;
        uint8_t *const st1 = smem + L.st1;
        uint8_t *const slots = smem + L.slots;
        R *const sH = reinterpret_cast<R *>(smem + L.heavy);
        const uint8_t *ent = STAGE ? smem + L.ent : reinterpret_cast<const uint8_t *>(a.ent) + (int64_t)ti.ent_off * kSlot;
        const uint8_t *act = STAGE ? smem + L.act : reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * kSlot;
        // incidence words of this tile: staged block, or the global table
        const uint16_t *incb = STAGE ? reinterpret_cast<const uint16_t *>(smem + L.inc) : a.inc;
        const uint32_t inc_base = STAGE ? (uint32_t)ti.inc_off : 0u;
        __syncthreads();  // the previous tile's last reads of shared memory are done

        for (int i = threadIdx.x; i < nm; i += blockDim.x) {
            const float4 *src = reinterpret_cast<const float4 *>(in + ((int64_t)ti.mass_off + i) * kRec);
#pragma unroll
            for (int v = 0; v < kRec / 16; v++) {
                const float4 x = __ldg(src + v);
                reinterpret_cast<float4 *>(st0 + (int64_t)i * kRec)[v] = x;
                reinterpret_cast<float4 *>(st1 + (int64_t)i * kRec)[v] = x;
            }
        }
        if constexpr (STAGE) {
            const float4 *ge = reinterpret_cast<const float4 *>(reinterpret_cast<const uint8_t *>(a.ent) +
                                                                (int64_t)ti.ent_off * kSlot);
            const float4 *ga = reinterpret_cast<const float4 *>(reinterpret_cast<const uint8_t *>(a.act) +
                                                                (int64_t)ti.ent_off * kSlot);
            for (int v = threadIdx.x; v < E * (kSlot / 16); v += blockDim.x)
                reinterpret_cast<float4 *>(smem + L.ent)[v] = __ldg(ge + v);
            for (int v = threadIdx.x; v < ti.nact * (kSlot / 16); v += blockDim.x)
                reinterpret_cast<float4 *>(smem + L.act)[v] = __ldg(ga + v);
            // inc_words is a multiple of 128 u16 words and inc_off of 4 (8-byte words)
            const uint2 *gi = reinterpret_cast<const uint2 *>(a.inc + ti.inc_off);
            for (int v = threadIdx.x; v < ti.inc_words / 4; v += blockDim.x)
                reinterpret_cast<uint2 *>(smem + L.inc)[v] = __ldg(gi + v);
        }
        if (threadIdx.x == 0) {  // the zero force padding codes name (slot E), never overwritten
            reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[0] = make_float4(0.f, 0.f, 0.f, 0.f);
            if constexpr (kSlot == 32)
                reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[1] = make_float4(0.f, 0.f, 0.f, 0.f);
        }

        // constants of this thread's masses (tile-local i = tid + k * blockDim)
        uint8_t fl[MPT];
        uint32_t d[MPT], woff[MPT];
        R mm[MPT];
#pragma unroll
        for (int k = 0; k < MPT; k++) {
            const int i = threadIdx.x + k * blockDim.x;
            fl[k] = MF_FIXED;
            d[k] = 0;
            woff[k] = 0;
            mm[k] = 1;
            if (i < nm) {
                const int64_t g = (int64_t)ti.mass_off + i;
                fl[k] = __ldg(a.flags + g);
                d[k] = __ldg(a.deg + g);
                mm[k] = __ldg(reinterpret_cast<const R *>(a.mass) + g);
                woff[k] = __ldg(a.warp_inc_off + ti.warp_off + (i >> 5)) - inc_base;
            }
        }
        __syncthreads();

        double T = T0;
        for (int64_t step = 0; step < nsteps; step++) {
            const StepTime tm = step_time(T);
            const int last = write_acc && step == nsteps - 1;
            const uint8_t *cur = (step & 1) ? st1 : st0;
            uint8_t *nxt = (step & 1) ? st0 : st1;

            // B: one force per slab entry
            for (int e = threadIdx.x; e < E; e += blockDim.x) {
                Rec16<PREC> rc, q{};
                if constexpr (STAGE) {
                    rc = load_rec<PREC>(ent + (int64_t)e * kSlot);
                    if (e < ti.nact) q = load_rec<PREC>(act + (int64_t)e * kSlot);
                } else {
                    rc = ldg_rec<PREC>(ent + (int64_t)e * kSlot);
                    if (e < ti.nact) q = ldg_rec<PREC>(act + (int64_t)e * kSlot);
                }
                entry_force<PREC>(rc, e < ti.nact, q, cur, tm, slots + (int64_t)e * kSlot);
            }
            __syncthreads();
            if (ti.nheavy > 0) {
                heavy_sums<PREC>(a, ti, slots, sH, threadIdx.x >> 5, nwarps);
                __syncthreads();
            }

            // C: per-mass gather and epilogue into the other buffer
#pragma unroll
            for (int k = 0; k < MPT; k++) {
                const int i = threadIdx.x + k * blockDim.x;
                if (i >= nm || (fl[k] & MF_FIXED)) continue;
                R F0 = 0, F1 = 0, F2 = 0;
                if (d[k] == 255) {
                    int h = 0;
                    while (h < ti.nheavy && a.heavy_local[ti.heavy_off + h] != i) h++;
                    F0 = F0 + sH[h];
                    F1 = F1 + sH[ti.nheavy + h];
                    F2 = F2 + sH[2 * ti.nheavy + h];
                } else if (d[k] > 0) {
                    const uint2 *ip = reinterpret_cast<const uint2 *>(incb + woff[k]) + (i & 31);
                    const uint32_t nw = (d[k] + 3) >> 2;
                    for (uint32_t w = 0; w < nw; w++) {
                        const uint2 cw = STAGE ? ip[32 * w] : __ldg(ip + 32 * w);
                        gather_word_padded<PREC>(slots, cw, F0, F1, F2);
                    }
                }
                St<PREC> s = load_state_smem<PREC>(cur, i);
                integrate<PREC, INTEG_EULER>(a, ti, (int64_t)ti.mass_off + i, fl[k], mm[k], F0, F1, F2, s, nxt, i,
                                             last, np, prm);
            }
            __syncthreads();
            T = T + prm->dt;
        }

        const uint8_t *fin = (nsteps & 1) ? st1 : st0;
        for (int i = threadIdx.x; i < nm; i += blockDim.x) {
#pragma unroll
            for (int v = 0; v < kRec / 16; v++)
                reinterpret_cast<float4 *>(out + ((int64_t)ti.mass_off + i) * kRec)[v] =
                    reinterpret_cast<const float4 *>(fin + (int64_t)i * kRec)[v];
        }
    }
}

template <int PREC, int STAGE>
const void *rt_kernel(int mpt) {
    switch (mpt) {
        case 1: return (const void *)k_tile_resident<PREC, 1, STAGE>;
        case 2: return (const void *)k_tile_resident<PREC, 2, STAGE>;
        default: return (const void *)k_tile_resident<PREC, 4, STAGE>;
    }
}

template <int PREC>
const void *rt_kernel(int mpt, int stage) {
    return stage ? rt_kernel<PREC, 1>(mpt) : rt_kernel<PREC, 0>(mpt);
}

const void *rt_kernel(int precision, int mpt, int stage) {
    return precision == P_FP64 ? rt_kernel<P_FP64>(mpt, stage)
           : precision == P_FP32 ? rt_kernel<P_FP32>(mpt, stage)
                                 : rt_kernel<P_FP32C>(mpt, stage);
}

// masses per thread rounds up to an instantiated count (1, 2, 4)
int rt_mpt(int mpt) { return mpt <= 1 ? 1 : (mpt <= 2 ? 2 : 4); }

}  // namespace

size_t tile_resident_smem_bytes(int precision, const TileInfo &ti, int stage) {
    return (size_t)rt_layout(precision, ti, stage).total;
}

cudaError_t tile_resident_prepare(int precision, int mpt, int stage, size_t smem) {
    if (mpt < 1 || mpt > kResMaxMpt) return cudaErrorInvalidValue;
    return raise_smem_limit(rt_kernel(precision, rt_mpt(mpt), stage), smem);
}

int tile_resident_ctas_per_sm(int precision, int mpt, int stage, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, rt_kernel(precision, rt_mpt(mpt), stage), threads, smem) !=
        cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_tile_resident(int precision, const StepArgs &a, const TileResArgs &r, int mpt, int threads,
                                 size_t smem, int parity, int64_t nsteps, int write_acc, cudaStream_t s) {
    if (nsteps <= 0 || r.ntiles <= 0) return cudaSuccess;
    if (mpt < 1 || mpt > kResMaxMpt) return cudaErrorInvalidValue;
    void *args[] = {const_cast<StepArgs *>(&a), const_cast<TileResArgs *>(&r), &parity, &nsteps, &write_acc};
    return cudaLaunchKernel(rt_kernel(precision, rt_mpt(mpt), r.stage), dim3(r.ntiles), dim3(threads), args, smem, s);
}

}  // namespace tg
