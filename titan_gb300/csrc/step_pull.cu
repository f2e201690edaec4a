// step_pull.cu -- pull form of the fused step (sm_103a), FP32 and FP32C.
//
// The slab forms compute each spring force once per tile into a
// shared-memory slot and gather the slots per mass; here every mass computes
// the forces of its own springs, in its incidence order, straight into its
// running sum: each spring is evaluated at both of its ends, which costs
// arithmetic (the kernel has plenty to spare) but takes the slot stores, the
// slot gathers, the slab records and the phase barrier out of shared memory.
// The force of a spring at its left end is exactly minus the force at its
// right end (pull_layout.h), so the sums -- and the states -- are the slab
// forms' bit for bit.
//
// One persistent CTA per SM:
//   * a producer warp walks the CTA's tiles (b, b + G, ...) and streams each
//     tile's state records into a ring of stages: the tile's own masses as
//     one bulk copy (TMA, cp.async.bulk), the halo masses as 16-byte
//     cp.async gathers from an index list that arrives one tile ahead, all
//     counted on the stage's "full" mbarrier;
//   * consumer warps form teams, one warp per 32 tile masses; team q takes
//     tiles q, q + nteams, ...  A warp streams its unit's spring columns
//     (pull_layout.h) from HBM straight into registers, one block of
//     kBlk columns ahead of the one it computes -- across tile boundaries,
//     so a new tile starts with its first columns already loaded -- waits
//     for its tile's stage, sums its springs' forces against the staged
//     states, integrates (epilogue.cuh) and releases the stage on its
//     "empty" mbarrier.
// Every wait is bounded: a time-out raises *err and the abort word, and the
// CTA waits (bounded) for its own copies in flight before it returns.
#include <cstdint>

#include "async_copy.cuh"
#include "engine.h"
#include "epilogue.cuh"
#include "grid_dep.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

constexpr int kPullThreads = (kPullMaxConsumerWarps + 1) * 32;
constexpr int kBlk = 8;  // spring columns per prefetched block

template <int PREC>
__host__ __device__ constexpr int pull_rec() { return PREC == P_FP32 ? 32 : 48; }

// One block of a lane's spring columns in registers.
struct ColBlock {
    uint32_t w[kBlk];
    float k[kBlk], r[kBlk];
};

// Where a warp's next block of columns comes from: tile t (its unit's block
// at base), block blk of nblk; deg is this lane's degree in that tile.
struct ColCursor {
    int t, blk, nblk, deg;
    const uint8_t *base;
    uint32_t wb, cs;  // words bytes, bytes of one column array (ncols * 128)
};

__device__ __forceinline__ void cursor_tile(const StepArgs &a, ColCursor &c, int u, int lane) {
    c.blk = 0;
    c.nblk = 0;
    c.deg = 0;
    const TileInfo &ti = a.tiles[c.t];
    const int nm = __ldg(&ti.nm);
    if (32 * u >= nm) return;
    const PullUnit pu = a.pull_units[__ldg(&ti.pad0) + u];
    c.nblk = (pu.ncols + kBlk - 1) / kBlk;
    c.base = a.pull_ell + (uint64_t)pu.ell * 128u;
    c.wb = pull_words_bytes(pu.ncols);
    c.cs = (uint32_t)pu.ncols * 128u;
    const int i = 32 * u + lane;
    if (i < nm) c.deg = __ldg(a.deg + __ldg(&ti.mass_off) + i);
}

// Moves the cursor to the warp's next block (skipping tiles where the warp
// has no masses); t >= ntiles marks the end.
__device__ __forceinline__ void cursor_next(const StepArgs &a, ColCursor &c, int stride, int u, int lane) {
    if (++c.blk < c.nblk) return;
    for (;;) {
        c.t += stride;
        if (c.t >= a.ntiles) {
            c.nblk = 0;
            return;
        }
        cursor_tile(a, c, u, lane);
        if (c.nblk > 0) return;
    }
}

// The block at the cursor (columns past the lane's degree are not read).
__device__ __forceinline__ void load_block(const ColCursor &c, int ntiles, int lane, ColBlock &b) {
    const bool any = c.t < ntiles && c.nblk > 0;
#pragma unroll
    for (int q = 0; q < kBlk; q++) {
        const int j = c.blk * kBlk + q;
        b.w[q] = 0;
        b.k[q] = 0.f;
        b.r[q] = 0.f;
        if (any && j < c.deg) {
            const uint8_t *p = c.base + (uint32_t)j * 64u + 2u * lane;
            b.w[q] = __ldcs(reinterpret_cast<const unsigned short *>(p));
            const uint8_t *pk = c.base + c.wb + (uint32_t)j * 128u + 4u * lane;
            b.k[q] = __ldcs(reinterpret_cast<const float *>(pk));
            b.r[q] = __ldcs(reinterpret_cast<const float *>(pk + c.cs));
        }
    }
}

// Adds the force of one spring on this mass (self: xs, xl, vs -- hi
// positions, lo positions, hi velocities) from the neighbour's state record
// staged at slot nbr: e = x_nbr - x_self (compensated in FP32C), and the
// sum receives -(e * fr) -- the slab forms' right-end force d * fr with
// d = -e, or minus their left-end force d * fr with d = e, the same value.
// The operations, their order and their roundings are spring_force's
// (tile_phases.cuh) with d replaced by e (exactly d or -d) and the damping
// velocity difference taken self minus neighbour (exactly v_l - v_r or its
// negation, so each product w_i e_i equals the slab forms').
template <int PREC>
__device__ __forceinline__ void pull_force(const float (&xs)[3], const float (&xl)[3], const float (&vs)[3],
                                           const uint8_t *st, uint32_t nbr, float k, float rest, float c,
                                           bool actuated, const float4 &act, const StepTime &t, float &F0,
                                           float &F1, float &F2) {
    constexpr int kV = PREC == P_FP32 ? 2 : 3;  // float4 per state record
    const float4 *pn = reinterpret_cast<const float4 *>(st) + nbr * kV;
    const float4 n0 = pn[0], n1 = pn[1];
    float e0 = n0.x - xs[0], e1 = n0.y - xs[1], e2 = n0.z - xs[2];
    if constexpr (PREC == P_FP32C) {
        const float n2x = reinterpret_cast<const float *>(pn + 2)[0];
        e0 += n1.z - xl[0];
        e1 += n1.w - xl[1];
        e2 += n2x - xl[2];
    }
    float rs = rest;
    if (actuated) {
        const float cyc = fmaf(act.x, t.hi, fmaf(act.x, t.lo, act.z));
        const float fr = cyc - rintf(cyc);
        rs = rest * fmaf(act.y, __sinf(6.28318530717958647692f * fr), 1.0f);
    }
    const float n2 = fmaf(e2, e2, fmaf(e1, e1, e0 * e0));
    float rq = rsqrtf(n2);
    rq = rq * fmaf(-0.5f * n2 * rq, rq, 1.5f);  // one Newton step
    const float nrm = n2 * rq;
    float f = k * (rs - nrm);
    if (c != 0.f) {
        const float w0 = vs[0] - n0.w, w1 = vs[1] - n1.x, w2 = vs[2] - n1.y;
        f = fmaf(fmaf(w2, e2, fmaf(w1, e1, w0 * e0)), rq * c, f);
    }
    const float fr = f * rq;
    F0 = F0 - e0 * fr;
    F1 = F1 - e1 * fr;
    F2 = F2 - e2 * fr;
}

template <int PREC, int INTEG>
__global__ void __launch_bounds__(kPullThreads, 1) k_step_pull(StepArgs a, int parity, int write_acc) {
    constexpr int kRec = pull_rec<PREC>();
    extern __shared__ __align__(128) uint8_t smem[];
    const PullLayout &L = a.pull;
    const int NS = L.nstages, NT = L.nteams, TW = L.team_warps;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + L.mbar);
    uint64_t *empty = full + NS;
    uint64_t *idxbar = empty + NS;  // [2]
    volatile int *abort_word = reinterpret_cast<volatile int *>(idxbar + 2);
    int *issued_word = reinterpret_cast<int *>(idxbar + 2) + 1;  // tiles whose copies were issued
    int *idx_issued = issued_word + 1, *idx_waited = issued_word + 2;
    int32_t *idxbuf = reinterpret_cast<int32_t *>(smem + L.idx);  // 2 * L.idx_words
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    DevParams *prm = reinterpret_cast<DevParams *>(smem + L.params);
    for (int q = threadIdx.x; q < (int)(sizeof(DevParams) / 16); q += blockDim.x)
        reinterpret_cast<int4 *>(prm)[q] = __ldg(reinterpret_cast<const int4 *>(a.prm) + q);
    // the next step's grid may launch now; before its grid_dep_wait() it
    // reads only data no step writes (spring columns, tile records)
    grid_dep_launch_dependents();
    const int ncw = NT * TW;  // consumer warps; the producer is warp ncw
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = gridDim.x;
    const int ntiles = a.ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 33);  // expect-tx arrival + one cp.async arrival per producer lane
            mbar_init(&empty[s], (uint32_t)TW);
        }
        mbar_init(&idxbar[0], 1);
        mbar_init(&idxbar[1], 1);
        *abort_word = 0;
        *issued_word = 0;
        *idx_issued = 0;
        *idx_waited = 0;
        fence_mbar_init();
    }
    __syncthreads();

    if (warp == ncw) {
        // ---------------- producer warp ----------------
        constexpr int kChunks = kRec / 16;
        auto issue_idx = [&](int j, const TileInfo &tj) {
            const uint32_t b = (uint32_t)((tj.nh + 3) & ~3) * 4u;
            fence_proxy_async();
            mbar_expect_tx(&idxbar[j & 1], b);
            issue_chunks(reinterpret_cast<uint8_t *>(idxbuf + (j & 1) * L.idx_words),
                         reinterpret_cast<const uint8_t *>(a.halo + tj.halo_off), b, &idxbar[j & 1]);
            *idx_issued = j + 1;
        };
        TileInfo ti = {};
        if (blockIdx.x < ntiles) ti = a.tiles[blockIdx.x];
        if (lane == 0 && blockIdx.x < ntiles) issue_idx(0, ti);
        int k = 0;
        for (int t = blockIdx.x; t < ntiles; t += G, k++) {
            const int s = k % NS;
            const uint32_t ph = (uint32_t)(k / NS) & 1u;
            const bool has_next = t + G < ntiles;
            TileInfo tn = {};
            if (has_next) tn = a.tiles[t + G];
            bool ok = bounded_wait(&empty[s], ph ^ 1u, abort_word, 200);
            if (ok) {
                ok = bounded_wait(&idxbar[k & 1], (uint32_t)(k >> 1) & 1u, abort_word);
                if (ok && lane == 0) *idx_waited = k + 1;
            }
            if (__any_sync(0xffffffffu, !ok || *abort_word)) {
                if (lane == 0) {
                    *abort_word = 1;
                    atomicOr(a.err, 1);
                }
                break;
            }
            uint8_t *st = smem + (int64_t)s * L.stage;
            // the state records are the previous step's output
            if (k == 0) grid_dep_wait();
            if (lane == 0) {
                fence_proxy_async();
                const uint32_t sb = (uint32_t)ti.nm * kRec;
                mbar_expect_tx(&full[s], sb);
                issue_chunks(st, in + (int64_t)ti.mass_off * kRec, sb, &full[s]);
            }
            const int32_t *ix = idxbuf + (k & 1) * L.idx_words;
            for (int h = lane; h < ti.nh; h += 32) {
                const uint8_t *src = in + (int64_t)ix[h] * kRec;
                uint8_t *dst = st + (int64_t)(ti.nm + h) * kRec;
#pragma unroll
                for (int c = 0; c < kChunks; c++) cp_async16(dst + 16 * c, src + 16 * c);
            }
            cp_async_arrive(&full[s]);
            __syncwarp();  // every lane has read ring entry k & 1
            if (lane == 0) {
                *issued_word = k + 1;
                if (has_next) issue_idx(k + 1, tn);
            }
            ti = tn;
        }
    } else if (warp < ncw) {
        // ---------------- consumer warps ----------------
        const int tm = warp / TW, u = warp % TW;
        const int stride = NT * G;
        // first block of this warp's columns: constant across steps, so
        // loaded before the wait for the previous step
        ColCursor cur;
        cur.t = blockIdx.x + tm * G;
        cur.nblk = 0;
        if (cur.t < ntiles) {
            cursor_tile(a, cur, u, lane);
            if (cur.nblk == 0) cursor_next(a, cur, stride, u, lane);
        }
        ColBlock blk;
        load_block(cur, ntiles, lane, blk);
        cursor_next(a, cur, stride, u, lane);
        grid_dep_wait();  // the time record is the previous step's output
        const StepTime tms = step_time(a.tbuf[parity]);
        if (threadIdx.x == 0 && blockIdx.x == 0) a.tbuf[parity ^ 1] = tms.T + a.prm->launch_dt;

        for (int k = tm, t = blockIdx.x + tm * G; t < ntiles; k += NT, t += stride) {
            const int s = k % NS;
            const uint32_t ph = (uint32_t)(k / NS) & 1u;
            const TileInfo &tg_ = a.tiles[t];
            const int nm = __ldg(&tg_.nm), mass_off = __ldg(&tg_.mass_off);
            const int i = 32 * u + lane;
            const bool unit = 32 * u < nm;
            PullUnit pu = {};
            if (unit) pu = a.pull_units[__ldg(&tg_.pad0) + u];
            const int nblk = unit ? (pu.ncols + kBlk - 1) / kBlk : 0;
            const bool ok = bounded_wait(&full[s], ph, abort_word);
            if (__any_sync(0xffffffffu, !ok)) {
                if (lane == 0) {
                    *abort_word = 1;
                    atomicOr(a.err, 1);
                }
                break;
            }
            const uint8_t *st = smem + (int64_t)s * L.stage;
            const bool active = i < nm;
            const int64_t g = (int64_t)mass_off + i;
            uint8_t fl = MF_FIXED;
            int deg = 0;
            float xs[3] = {0.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f}, vs[3] = {0.f, 0.f, 0.f};
            if (active) {
                fl = __ldg(a.flags + g);
                deg = __ldg(a.deg + g);
                const St<PREC> sv = load_state_smem<PREC>(st, i);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    xs[q] = sv.x[q];
                    xl[q] = sv.xl[q];
                    vs[q] = sv.v[q];
                }
            }
            // this lane's actuation records, one prefetched ahead
            const float4 *actp = nullptr;
            int nact = 0;
            float4 actn = make_float4(0.f, 0.f, 0.f, 0.f);
            if (active && deg > 0) {
                const unsigned short *off =
                    reinterpret_cast<const unsigned short *>(a.pull_act + pu.act);
                const int o0 = __ldg(off + lane), o1 = __ldg(off + lane + 1);
                actp = a.pull_act + pu.act + kPullActHeader + o0;
                nact = o1 - o0;
                if (nact > 0) actn = __ldg(actp);
            }
            const bool col_damp = (pu.flags & PU_DAMP) != 0;
            const float cu = pu.damping;
            const uint8_t *dbase = a.pull_ell + (uint64_t)pu.ell * 128u + pull_words_bytes(pu.ncols) +
                                   2u * (uint32_t)pu.ncols * 128u + 4u * lane;
            float F0 = 0.f, F1 = 0.f, F2 = 0.f;
            for (int b = 0; b < nblk; b++) {
                ColBlock nxt;
                load_block(cur, ntiles, lane, nxt);
                cursor_next(a, cur, stride, u, lane);
#pragma unroll
                for (int q = 0; q < kBlk; q++) {
                    const int j = b * kBlk + q;
                    if (j < deg) {
                        const uint32_t w = blk.w[q];
                        const bool act = (w & 0x8000u) != 0;
                        float4 ar = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (act) {
                            ar = actn;
                            ++actp;
                            if (--nact > 0) actn = __ldg(actp);
                        }
                        const float c = col_damp ? __ldg(reinterpret_cast<const float *>(dbase + (uint32_t)j * 128u))
                                                 : cu;
                        pull_force<PREC>(xs, xl, vs, st, w & 0xfffu, blk.k[q], blk.r[q], c, act, ar, tms, F0, F1,
                                         F2);
                    }
                }
                blk = nxt;
            }
            if (active && !(fl & MF_FIXED)) {  // src/sim.cu:1100
                // the whole record again (the stage is held until the arrival below)
                St<PREC> sv = load_state_smem<PREC>(st, i);
                TileInfo ti;
                ti.body = __ldg(&tg_.body);
                const float m = __ldg(reinterpret_cast<const float *>(a.mass) + g);
                integrate<PREC, INTEG>(a, ti, g, fl, m, F0, F1, F2, sv, out, g, write_acc, np, prm);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    }

    // drain: after an abort, the copies issued for the last stages may still
    // be in flight; each stage's last use is one of the last NS issued tiles
    __syncthreads();
    if (threadIdx.x == 0) {
        const int issued = *issued_word;
        for (int k = issued - NS > 0 ? issued - NS : 0; k < issued; k++) {
            const int s = k % NS;
            const uint32_t ph = (uint32_t)(k / NS) & 1u;
            for (uint32_t it = 0; it < kWaitLimit && !mbar_try_wait(&full[s], ph); it++) {
            }
        }
        for (int j = *idx_waited; j < *idx_issued; j++)
            for (uint32_t it = 0; it < kWaitLimit && !mbar_try_wait(&idxbar[j & 1], (uint32_t)(j >> 1) & 1u); it++) {
            }
    }
}

template <int PREC>
const void *pull_kernel(int integ) {
    switch (integ) {
        case INTEG_VERLET: return (const void *)k_step_pull<PREC, INTEG_VERLET>;
        case INTEG_RK2: return (const void *)k_step_pull<PREC, INTEG_RK2>;
        default: return (const void *)k_step_pull<PREC, INTEG_EULER>;
    }
}

const void *pull_kernel(int precision, int integ) {
    return precision == P_FP32 ? pull_kernel<P_FP32>(integ) : pull_kernel<P_FP32C>(integ);
}

}  // namespace

cudaError_t step_pull_prepare(int precision, int integ, size_t smem) {
    if (precision == P_FP64) return cudaErrorInvalidValue;
    return raise_smem_limit(pull_kernel(precision, integ), smem);
}

cudaError_t launch_step_pull(int precision, int integ, const StepArgs &a, int ctas, int parity, int write_acc,
                             cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    const int ncw = a.pull.nteams * a.pull.team_warps;
    if (precision == P_FP64 || ncw < 1 || ncw > kPullMaxConsumerWarps || a.pull.nstages < a.pull.nteams ||
        a.pull.nstages % a.pull.nteams || a.pull.nstages > kPullMaxStages)
        return cudaErrorInvalidValue;
    void *args[] = {const_cast<StepArgs *>(&a), &parity, &write_acc};
    return launch_programmatic(pull_kernel(precision, integ), dim3(ctas), dim3((ncw + 1) * 32), args,
                               (size_t)a.pull.total, s);
}

}  // namespace tg
