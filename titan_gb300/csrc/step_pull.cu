// step_pull.cu -- pull form of the fused step (sm_103a), FP32 and FP32C.
//
// The slab forms compute each spring force once per tile into a
// shared-memory slot and gather the slots per mass; here every mass computes
// the forces of its own springs, in its incidence order, straight into its
// running sum: each spring is evaluated at both of its ends, which costs
// arithmetic but takes the slot stores, the slot gathers, the slab records
// and the phase barrier out of shared memory.  The force of a spring at its
// left end is exactly minus the force at its right end (pull_layout.h), so
// the sums -- and the states -- are the slab forms' bit for bit.
//
// One persistent CTA per SM:
//   * a producer warp walks the CTA's tiles (b, b + G, ...) and streams each
//     tile into a ring of stages: the tile's own state records as one bulk
//     copy (TMA, cp.async.bulk), the tile's actuation records as another,
//     and the halo masses' records as 16-byte cp.async gathers from an index
//     list that arrives one tile ahead, all counted on the stage's "full"
//     mbarrier;
//   * consumer warps form teams, one warp per 32 tile masses (a unit); team
//     q takes tiles q, q + nteams, ...  A warp streams its units' spring
//     columns (pull_layout.h), four columns per 8- and 16-byte vector loads,
//     from HBM into registers kAhead quads ahead of the quad it computes --
//     across tile boundaries, with each next unit's descriptor loaded a tile
//     ahead -- waits for its tile's stage, sums its springs' forces against
//     the staged states, integrates (epilogue.cuh) and releases the stage on
//     its "empty" mbarrier.
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

template <int PREC>
__host__ __device__ constexpr int pull_rec() { return PREC == P_FP32 ? 32 : 48; }

// One quad of a lane's spring columns in registers.
struct Quad {
    uint2 w;
    float4 k, r;
};

__device__ __forceinline__ void load_quad(const uint8_t *qp, int lane, Quad &d) {
    d.w = __ldcs(reinterpret_cast<const uint2 *>(qp + 8 * lane));
    d.k = __ldcs(reinterpret_cast<const float4 *>(qp + 256 + 16 * lane));
    d.r = __ldcs(reinterpret_cast<const float4 *>(qp + 768 + 16 * lane));
}

__device__ __forceinline__ PullUnit load_unit(const StepArgs &a, int t, int u) {
    PullUnit pu;
    *reinterpret_cast<int4 *>(&pu) =
        __ldg(reinterpret_cast<const int4 *>(a.pull_units) + (int64_t)t * a.pull.team_warps + u);
    return pu;
}

// The warp's stream of quads: quad q of its unit pu in tile t; pn is its
// unit in the tile after (loaded a tile ahead).  t >= ntiles: the end.
struct QuadCursor {
    int t, q, stride;
    PullUnit pu, pn;
};

__device__ __forceinline__ void cursor_tile(const StepArgs &a, QuadCursor &c, int u) {
    c.t += c.stride;
    c.pu = c.pn;
    if (c.t + c.stride < a.ntiles) c.pn = load_unit(a, c.t + c.stride, u);
}

// Moves to the warp's next quad, skipping tiles where its unit has none.
__device__ __forceinline__ void cursor_next(const StepArgs &a, QuadCursor &c, int u) {
    if (++c.q < c.pu.nquads) return;
    c.q = 0;
    do {
        cursor_tile(a, c, u);
    } while (c.t < a.ntiles && c.pu.nquads == 0);
}

__device__ __forceinline__ void cursor_load(const StepArgs &a, const QuadCursor &c, int lane, Quad &d) {
    if (c.t < a.ntiles)
        load_quad(a.pull_ell + (uint64_t)c.pu.ell * 128u + (uint32_t)c.q * pull_quad_bytes(c.pu.flags & PU_DAMP),
                  lane, d);
}

// Named-barrier OR over a team (bar.red.or: every thread of the team takes
// part and receives the same answer).
__device__ __forceinline__ bool team_any(int id, int nthreads, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void team_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// The four columns of quad Q, summed into F in column order.  Each column
// is one spring of this mass (self: xs, xl, vs -- hi positions, lo
// positions, hi velocities) and the neighbour's state record in the stage
// (st4, a float4 index in the word): e = x_nbr - x_self (compensated in
// FP32C), and the sum receives -(e * fr) -- the slab forms' right-end force
// d * fr with d = -e, or minus their left-end force d * fr with d = e, the
// same value.  The operations, their order and their roundings are
// spring_force's (tile_phases.cuh) with d replaced by e (exactly d or -d)
// and the damping velocity difference taken self minus neighbour (exactly
// v_l - v_r or its negation, so each product w_i e_i equals the slab
// forms').  An actuated column's rest length is the rest' its tile's team
// computed into the stage (act[e].w).  The four columns run as straight-line
// code (so their chains interleave); a padding column computes garbage from
// slot 0 and adds fr = 0: subtracting e * 0 = +0 leaves any running sum's
// bits unchanged, as skipping it would.  DAMP: the damping term, whose
// c = 0 columns (per-column damping) likewise change no bits.
template <int PREC, bool DAMP>
__device__ __forceinline__ void pull_quad(const Quad &Q, const float4 *st4, const float4 *act, const float (&xs)[3],
                                          const float (&xl)[3], const float (&vs)[3], float4 dq, float &F0,
                                          float &F1, float &F2) {
    const float kq[4] = {Q.k.x, Q.k.y, Q.k.z, Q.k.w};
    const float rq4[4] = {Q.r.x, Q.r.y, Q.r.z, Q.r.w};
    const float cq[4] = {dq.x, dq.y, dq.z, dq.w};
    float p0[4], p1[4], p2[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const uint32_t w = ((c < 2 ? Q.w.x : Q.w.y) >> (16 * (c & 1))) & 0xffffu;
        const float rs = (w & PW_ACT) ? act[__float_as_uint(rq4[c])].w : rq4[c];
        const float4 *pn = st4 + (w & PW_SLOT);
        const float4 n0 = pn[0], n1 = pn[1];
        float e0 = n0.x - xs[0], e1 = n0.y - xs[1], e2 = n0.z - xs[2];
        if constexpr (PREC == P_FP32C) {
            const float n2x = reinterpret_cast<const float *>(pn + 2)[0];
            e0 += n1.z - xl[0];
            e1 += n1.w - xl[1];
            e2 += n2x - xl[2];
        }
        const float n2 = fmaf(e2, e2, fmaf(e1, e1, e0 * e0));
        float rq = rsqrtf(n2);
        rq = rq * fmaf(-0.5f * n2 * rq, rq, 1.5f);  // one Newton step
        const float nrm = n2 * rq;
        float f = kq[c] * (rs - nrm);
        if constexpr (DAMP) {
            const float w0 = vs[0] - n0.w, w1 = vs[1] - n1.x, w2 = vs[2] - n1.y;
            f = fmaf(fmaf(w2, e2, fmaf(w1, e1, w0 * e0)), rq * cq[c], f);
        }
        const float fr = (w & PW_VALID) ? f * rq : 0.f;
        p0[c] = e0 * fr;
        p1[c] = e1 * fr;
        p2[c] = e2 * fr;
    }
#pragma unroll
    for (int c = 0; c < 4; c++) {
        F0 = F0 - p0[c];
        F1 = F1 - p1[c];
        F2 = F2 - p2[c];
    }
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
                const uint32_t sb = (uint32_t)ti.nm * kRec, ab = (uint32_t)ti.nact * 16u;
                mbar_expect_tx(&full[s], sb + ab);
                // the actuation records: constant, read once per step
                issue_chunks_hint(st + L.act_off, reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * 16,
                                  ab, &full[s], l2_evict_first_policy());
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
        const int bar_id = 1 + tm, team_threads = TW * 32;  // the team's named barrier
        const int t0 = blockIdx.x + tm * G;
        // the quad stream, kAhead = 2 quads ahead of the computed one, in
        // buffers A and B taking turns (qa: the next quad to compute is in A);
        // spring columns are constant across steps, so the first quads are
        // loaded before the wait for the previous step
        QuadCursor cur;
        cur.t = t0 - stride;
        cur.q = 0;
        cur.stride = stride;
        cur.pn = PullUnit{};
        if (t0 < ntiles) cur.pn = load_unit(a, t0, u);
        do {
            cursor_tile(a, cur, u);
        } while (cur.t < ntiles && cur.pu.nquads == 0);
        Quad qa{}, qb{};
        cursor_load(a, cur, lane, qa);
        if (cur.t < ntiles) cursor_next(a, cur, u);
        cursor_load(a, cur, lane, qb);
        if (cur.t < ntiles) cursor_next(a, cur, u);
        bool in_a = true;
        // this warp's unit, and the tile's actuated entries and body, in the
        // tile it computes next
        PullUnit upn = PullUnit{};
        int nact_n = 0, body_n = 0;
        if (t0 < ntiles) {
            upn = load_unit(a, t0, u);
            nact_n = __ldg(&a.tiles[t0].nact);
            body_n = __ldg(&a.tiles[t0].body);
        }
        grid_dep_wait();  // the time record is the previous step's output
        const StepTime tms = step_time(a.tbuf[parity]);
        if (threadIdx.x == 0 && blockIdx.x == 0) a.tbuf[parity ^ 1] = tms.T + a.prm->launch_dt;

        for (int k = tm, t = t0; t < ntiles; k += NT, t += stride) {
            const int s = k % NS;
            const uint32_t ph = (uint32_t)(k / NS) & 1u;
            const PullUnit pu = upn;
            const int nact = nact_n, body = body_n;
            if (t + stride < ntiles) {
                upn = load_unit(a, t + stride, u);
                nact_n = __ldg(&a.tiles[t + stride].nact);
                body_n = __ldg(&a.tiles[t + stride].body);
            }
            const bool active = lane < pu.lanes;
            const int64_t g = (int64_t)pu.mass0 + lane;
            uint8_t fl = MF_FIXED;
            float m = 1.f;
            if (active) {  // used in the epilogue: loaded now
                fl = __ldg(a.flags + g);
                m = __ldg(reinterpret_cast<const float *>(a.mass) + g);
            }
            const bool ok = bounded_wait(&full[s], ph, abort_word);
            const uint8_t *st = smem + (int64_t)s * L.stage;
            const float4 *st4 = reinterpret_cast<const float4 *>(st);
            float4 *act = reinterpret_cast<float4 *>(const_cast<uint8_t *>(st) + L.act_off);
            // rest' of the tile's actuated springs (its first nact slab
            // entries), once per tile: rest (1 + a sin(2 pi frac(nu T + phi)))
            // as the slab forms compute it, over the record's rest
            if (ok) {
                for (int e = u * 32 + lane; e < nact; e += team_threads) {
                    const float4 q = act[e];
                    const float cyc = fmaf(q.x, tms.hi, fmaf(q.x, tms.lo, q.z));
                    const float fr = cyc - rintf(cyc);
                    act[e].w = q.w * fmaf(q.y, __sinf(6.28318530717958647692f * fr), 1.0f);
                }
            }
            // one team barrier: orders the rest' stores before their reads and
            // makes a time-out the whole team's decision
            if (team_any(bar_id, team_threads, !ok)) {
                if (lane == 0) {
                    *abort_word = 1;
                    atomicOr(a.err, 1);
                }
                break;
            }
            float xs[3] = {0.f, 0.f, 0.f}, xl[3] = {0.f, 0.f, 0.f}, vs[3] = {0.f, 0.f, 0.f};
            if (active) {
                const St<PREC> sv = load_state_smem<PREC>(st, 32 * u + lane);
#pragma unroll
                for (int q = 0; q < 3; q++) {
                    xs[q] = sv.x[q];
                    xl[q] = sv.xl[q];
                    vs[q] = sv.v[q];
                }
            }
            const bool col_damp = (pu.flags & PU_DAMP) != 0;
            const bool damped = col_damp || pu.damping != 0.f;
            const float cu = pu.damping;
            const uint8_t *qbase = a.pull_ell + (uint64_t)pu.ell * 128u + 1280u + 16u * lane;
            float F0 = 0.f, F1 = 0.f, F2 = 0.f;
            for (int qi = 0; qi < pu.nquads; qi++) {
                float4 dq = make_float4(cu, cu, cu, cu);
                if (col_damp) dq = __ldg(reinterpret_cast<const float4 *>(qbase + (uint32_t)qi * 1792u));
                if (in_a) {
                    if (damped)
                        pull_quad<PREC, true>(qa, st4, act, xs, xl, vs, dq, F0, F1, F2);
                    else
                        pull_quad<PREC, false>(qa, st4, act, xs, xl, vs, dq, F0, F1, F2);
                    cursor_load(a, cur, lane, qa);
                } else {
                    if (damped)
                        pull_quad<PREC, true>(qb, st4, act, xs, xl, vs, dq, F0, F1, F2);
                    else
                        pull_quad<PREC, false>(qb, st4, act, xs, xl, vs, dq, F0, F1, F2);
                    cursor_load(a, cur, lane, qb);
                }
                if (cur.t < ntiles) cursor_next(a, cur, u);
                in_a = !in_a;
            }
            if (active && !(fl & MF_FIXED)) {  // src/sim.cu:1100
                // the whole record again (the stage is held until the arrival below)
                St<PREC> sv = load_state_smem<PREC>(st, 32 * u + lane);
                TileInfo ti;
                ti.body = body;
                integrate<PREC, INTEG>(a, ti, g, fl, m, F0, F1, F2, sv, out, g, write_acc, np, prm);
            }
            // the stage is free once every warp of the team is past it; order
            // this warp's rest' stores before the copies that will reuse it
            fence_proxy_async();
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
