// resident.cu -- batched bodies, all steps in one persistent launch.
//
// For a batch of independent soft bodies (set_bodies), the bodies that fit
// one CTA are packed into bins (plan.h ResPlan).  A CTA takes the next bin
// from a queue, stages its masses' state records in shared memory twice
// (current and next state), and runs every requested step there: per mass,
// the forces of its springs in ascending spring order, then the per-mass
// epilogue, the new state going to the other buffer; one barrier per step.
// Spring and actuation records stream from L2; the state leaves shared
// memory only once, after the last step.
//
// Each spring's force is evaluated at both of its ends (no force slots, so
// shared memory holds the state alone) by spring_force (tile_phases.cuh),
// the function the tiled kernels use, from the same endpoint states, and
// summed in the same order: results are bit-identical to the per-step
// kernels, and in FP64 to the CPU oracle.
#include <cstdint>

#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

constexpr int kResPf = 2;  // spring records in flight per mass

template <int PREC>
__host__ __device__ constexpr int res_rec_bytes() { return PREC == P_FP32 ? 32 : 48; }

template <int PREC, int MPT>
__global__ void __launch_bounds__(512) k_resident(StepArgs a, ResArgs r, int parity, int64_t nsteps, int write_acc) {
    using R = typename Real<PREC>::T;
    constexpr int kRec = res_rec_bytes<PREC>();
    constexpr int kEnt = PREC == P_FP64 ? 32 : 16;
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_bin;
    uint8_t *const st0 = smem;
    uint8_t *const st1 = smem + (int64_t)r.cap * kRec;
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    uint8_t *out = reinterpret_cast<uint8_t *>((parity ^ (int)(nsteps & 1)) ? a.state1 : a.state0);
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const double T0 = a.tbuf[parity];
    const double dt = prm->dt;
    const uint8_t *recs = reinterpret_cast<const uint8_t *>(r.rec);
    const uint8_t *acts = reinterpret_cast<const uint8_t *>(r.act);

    for (;;) {
        if (threadIdx.x == 0) s_bin = atomicAdd(r.next, 1);
        __syncthreads();
        const int bin = s_bin;
        if (bin >= r.nbins) break;
        const int64_t m0 = r.bin_mass_off[bin];
        const int nm = (int)(r.bin_mass_off[bin + 1] - m0);
        const int64_t w0 = r.bin_warp_off[bin];

        // constants of this thread's masses (bin-local i = tid + k * blockDim)
        int32_t g[MPT], bd[MPT];
        uint32_t d[MPT], ro[MPT];
        uint8_t fl[MPT];
        uint64_t am[MPT];
        R mm[MPT];
#pragma unroll
        for (int k = 0; k < MPT; k++) {
            const int i = threadIdx.x + k * blockDim.x;
            g[k] = 0;
            bd[k] = 0;
            d[k] = 0;
            ro[k] = 0;
            fl[k] = MF_FIXED;
            am[k] = 0;
            mm[k] = 1;
            if (i < nm) {
                g[k] = __ldg(r.mass + m0 + i);
                fl[k] = __ldg(a.flags + g[k]);
                d[k] = __ldg(r.deg + m0 + i);
                am[k] = __ldg(reinterpret_cast<const unsigned long long *>(r.act_mask) + m0 + i);
                ro[k] = __ldg(r.warp_rec_off + w0 + (i >> 5)) + (i & 31);
                mm[k] = __ldg(reinterpret_cast<const R *>(a.mass) + g[k]);
                if (fl[k] & MF_BODYPLANE) bd[k] = __ldg(r.body + m0 + i);
                const float4 *src = reinterpret_cast<const float4 *>(in + (int64_t)g[k] * kRec);
#pragma unroll
                for (int v = 0; v < kRec / 16; v++) {
                    const float4 x = __ldg(src + v);
                    reinterpret_cast<float4 *>(st0 + (int64_t)i * kRec)[v] = x;
                    reinterpret_cast<float4 *>(st1 + (int64_t)i * kRec)[v] = x;
                }
            }
        }
        __syncthreads();

        double T = T0;
        for (int64_t step = 0; step < nsteps; step++) {
            const StepTime tm = step_time(T);
            const int last = write_acc && step == nsteps - 1;
            const uint8_t *cur = (step & 1) ? st1 : st0;
            uint8_t *nxt = (step & 1) ? st0 : st1;
#pragma unroll
            for (int k = 0; k < MPT; k++) {
                const int i = threadIdx.x + k * blockDim.x;
                if (i >= nm || (fl[k] & MF_FIXED)) continue;
                R F0 = 0, F1 = 0, F2 = 0;
                const uint32_t dk = d[k];
                const uint8_t *rp = recs + (int64_t)ro[k] * kEnt;
                const uint8_t *ap = acts + (int64_t)ro[k] * kEnt;
                Rec16<PREC> rq[kResPf], aq[kResPf] = {};
#pragma unroll
                for (int p = 0; p < kResPf; p++) {
                    if ((uint32_t)p < dk) {
                        rq[p] = ldg_rec<PREC>(rp + (int64_t)p * 32 * kEnt);
                        if ((am[k] >> p) & 1) aq[p] = ldg_rec<PREC>(ap + (int64_t)p * 32 * kEnt);
                    }
                }
                for (uint32_t j = 0; j < dk; j += kResPf) {
#pragma unroll
                    for (int p = 0; p < kResPf; p++) {
                        const uint32_t jj = j + p;
                        if (jj >= dk) break;
                        const Rec16<PREC> rc = rq[p];
                        const Rec16<PREC> ac = aq[p];
                        const uint32_t jn = jj + kResPf;
                        if (jn < dk) {
                            rq[p] = ldg_rec<PREC>(rp + (int64_t)jn * 32 * kEnt);
                            if (jn >= 64 || ((am[k] >> jn) & 1))
                                aq[p] = ldg_rec<PREC>(ap + (int64_t)jn * 32 * kEnt);
                        }
                        uint32_t word;
                        R ks, rest, damp;
                        if constexpr (PREC == P_FP64) {
                            word = (uint32_t)__double_as_longlong(rc.hi.y);
                            ks = rc.lo.x;
                            rest = rc.lo.y;
                            damp = rc.hi.x;
                        } else {
                            word = __float_as_uint(rc.v.x);
                            ks = rc.v.y;
                            rest = rc.v.z;
                            damp = rc.v.w;
                        }
                        const int other = (int)(word & 0x7fffu);
                        const bool right = (word & 0x8000u) != 0;
                        const uint32_t type = (word >> 16) & 3u;
                        const F3<PREC> f = spring_force<PREC>(right ? other : i, right ? i : other, type, ks, rest,
                                                              damp, type >= 2, ac, cur, tm);
                        if constexpr (PREC == P_FP64) {
                            const double sg = right ? 1.0 : -1.0;
                            F0 = fma(sg, f.x, F0);
                            F1 = fma(sg, f.y, F1);
                            F2 = fma(sg, f.z, F2);
                        } else {
                            const float sg = right ? 1.0f : -1.0f;
                            F0 = fmaf(sg, f.x, F0);
                            F1 = fmaf(sg, f.y, F1);
                            F2 = fmaf(sg, f.z, F2);
                        }
                    }
                }
                TileInfo tb{};
                tb.body = bd[k];
                St<PREC> s = load_state_smem<PREC>(cur, i);
                integrate<PREC, INTEG_EULER>(a, tb, g[k], fl[k], mm[k], F0, F1, F2, s, nxt, i, last, np, prm);
            }
            __syncthreads();
            T = T + dt;
        }
        const uint8_t *fin = (nsteps & 1) ? st1 : st0;
#pragma unroll
        for (int k = 0; k < MPT; k++) {
            const int i = threadIdx.x + k * blockDim.x;
            if (i >= nm) continue;
#pragma unroll
            for (int v = 0; v < kRec / 16; v++)
                reinterpret_cast<float4 *>(out + (int64_t)g[k] * kRec)[v] =
                    reinterpret_cast<const float4 *>(fin + (int64_t)i * kRec)[v];
        }
    }
}

// Advances the device time record by nsteps additions of dt (the same
// additions the per-step kernels make), for launches with no per-step tiles.
__global__ void k_advance_time(double *tbuf, int parity, int64_t nsteps, const DevParams *prm) {
    double T = tbuf[parity];
    const double dt = prm->dt;
    for (int64_t k = 0; k < nsteps; k++) T = T + dt;
    tbuf[parity ^ (int)(nsteps & 1)] = T;
}

template <int PREC>
const void *res_kernel(int mpt) {
    switch (mpt) {
        case 1: return (const void *)k_resident<PREC, 1>;
        case 2: return (const void *)k_resident<PREC, 2>;
        case 3: return (const void *)k_resident<PREC, 3>;
        default: return (const void *)k_resident<PREC, 4>;
    }
}

const void *res_kernel(int precision, int mpt) {
    return precision == P_FP64 ? res_kernel<P_FP64>(mpt)
           : precision == P_FP32 ? res_kernel<P_FP32>(mpt)
                                 : res_kernel<P_FP32C>(mpt);
}

}  // namespace

size_t resident_smem_bytes(int precision, int cap) {
    return 2 * (size_t)cap * (size_t)(precision == P_FP32 ? 32 : 48);
}

cudaError_t resident_prepare(int precision, int mpt, size_t smem) {
    if (mpt < 1 || mpt > kResMaxMpt) return cudaErrorInvalidValue;
    return raise_smem_limit(res_kernel(precision, mpt), smem);
}

int resident_ctas_per_sm(int precision, int mpt, int threads, size_t smem) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, res_kernel(precision, mpt), threads, smem) != cudaSuccess)
        return 0;
    return n;
}

cudaError_t launch_resident(int precision, const StepArgs &a, const ResArgs &r, int ctas, int threads, int parity,
                            int64_t nsteps, int write_acc, int write_time, cudaStream_t s) {
    if (nsteps <= 0) return cudaSuccess;
    if (r.nbins > 0) {
        const int mpt = (r.cap + threads - 1) / threads;
        if (mpt < 1 || mpt > kResMaxMpt) return cudaErrorInvalidValue;
        cudaError_t e = cudaMemsetAsync(r.next, 0, sizeof(int), s);
        if (e != cudaSuccess) return e;
        const size_t smem = resident_smem_bytes(precision, r.cap);
        void *args[] = {const_cast<StepArgs *>(&a), const_cast<ResArgs *>(&r), &parity, &nsteps, &write_acc};
        e = cudaLaunchKernel(res_kernel(precision, mpt), dim3(ctas), dim3(threads), args, smem, s);
        if (e != cudaSuccess) return e;
    }
    return write_time ? launch_advance_time(a, parity, nsteps, s) : cudaSuccess;
}

cudaError_t launch_advance_time(const StepArgs &a, int parity, int64_t nsteps, cudaStream_t s) {
    k_advance_time<<<1, 1, 0, s>>>(a.tbuf, parity, nsteps, a.prm);
    return cudaGetLastError();
}

}  // namespace tg
