// step_ws.cu -- warp-specialised persistent form of the fused step (sm_103a).
//
// Same tiles, arithmetic, summation order and results as k_step
// (step_kernel.cuh) -- the tests check them bit for bit.  The per-tile forms
// alternate, inside each CTA, between waiting for a tile's data and
// computing on it; here the two run concurrently in one persistent CTA per
// SM:
//   * two producer warps walk the CTA's tiles (b, b + G, b + 2G, ...) and,
//     for each, wait until a stage of the shared-memory ring is free, then
//     stream the tile into it: the first issues the slab records (into the
//     force slots) and the tile masses' state records as bulk copies on the
//     Tensor Memory Accelerator, and both gather the halo state records as
//     16-byte cp.async copies, all counted on the stage's "full" mbarrier
//     (one expect-tx arrival plus one cp.async arrival per producer lane).
//     The halo gathers are what a consumer group waits for once its stage
//     is free, so two warps share them (one takes about 2,700 cycles per
//     tile of 208 masses).  The halo index
//     list of the next tile arrives by bulk copy into a two-entry ring while
//     the current tile is issued, so no gather waits on an index load;
//     The stage also receives the tile's actuation records and incidence
//     block, so consumers never wait on a global load for them;
//   * the consumer warps form two groups that take alternate tiles (while one
//     group is in its narrow per-mass phase, the other computes entry
//     forces).  A group waits for "full", computes each entry's force over
//     its record (phase B), sums each mass's incident slots in ascending
//     spring order and integrates (phase C), then releases the stage on its
//     "empty" mbarrier.
// Each group synchronises on its own named barrier (1 or 2).  Every wait is
// bounded; a time-out is made uniform within a group (bar.red.or), raises
// *err and the shared abort word, and the CTA drains its own copies
// (bounded) before it returns.
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

constexpr int kBatchB = 3;  // slab entries per thread in flight (phase B); 4 spills at the 128-register cap
constexpr int kWsThreads = (kWsMaxConsumerWarps + kWsProducerWarps) * 32;
constexpr int kProdThreads = kWsProducerWarps * 32;
constexpr int kProdBar = 3;  // named barrier of the producer warps (the groups use 1 and 2)

template <int PREC>
__host__ __device__ constexpr int ws_rec() { return PREC == P_FP32 ? 32 : 48; }

__device__ __forceinline__ void group_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
// Named-barrier OR over a consumer group.
__device__ __forceinline__ bool group_any(int id, int nthreads, bool v) {
    uint32_t r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, %3, p;\n selp.u32 %0, 1, 0, q;\n}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(nthreads)
        : "memory");
    return r != 0;
}

template <int PREC, int INTEG>
__global__ void __launch_bounds__(kWsThreads, 1) k_step_ws(StepArgs a, int parity, int write_acc) {
    using R = typename Real<PREC>::T;
    constexpr int kRec = ws_rec<PREC>();
    constexpr int kSlot = Slot<PREC>::kBytes;
    extern __shared__ __align__(128) uint8_t smem[];
    const WsLayout &L = a.ws;
    const int NS = L.nstages;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + L.mbar);
    uint64_t *empty = full + NS;
    uint64_t *idxbar = empty + NS;  // [2]
    volatile int *abort_word = reinterpret_cast<volatile int *>(idxbar + 2);
    int *issued_word = reinterpret_cast<int *>(idxbar + 2) + 1;  // tiles whose copies were issued
    int *idx_issued = issued_word + 1, *idx_waited = issued_word + 2;
    int *last_word = issued_word + 3;                              // [2]: last tile each group consumed
    int32_t *idxbuf = reinterpret_cast<int32_t *>(smem + L.idx);  // 2 * L.idx_words
    TileInfo *tinfo = reinterpret_cast<TileInfo *>(smem + L.tinfo);  // [NS]: the tile in each stage
    const uint8_t *in = reinterpret_cast<const uint8_t *>(parity ? a.state1 : a.state0);
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    // the step's parameters, read per mass by the epilogue, from shared memory
    DevParams *prm = reinterpret_cast<DevParams *>(smem + L.params);
    for (int q = threadIdx.x; q < (int)(sizeof(DevParams) / 16); q += blockDim.x)
        reinterpret_cast<int4 *>(prm)[q] = __ldg(reinterpret_cast<const int4 *>(a.prm) + q);
    // the next step's grid may launch now: its CTAs take SMs as this grid's
    // leave, and everything it does before its grid_dep_wait() reads only
    // data no step writes (see the producer and the consumers below)
    grid_dep_launch_dependents();
    const int ncw = (int)(blockDim.x >> 5) - kWsProducerWarps;  // consumer warps (even)
    const int gw = ncw >> 1;                     // warps per group
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int G = gridDim.x;
    const int ntiles = a.ntiles;

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; s++) {
            mbar_init(&full[s], 1 + kProdThreads);  // expect-tx arrival + one cp.async arrival per producer lane
            mbar_init(&empty[s], (uint32_t)gw);
        }
        mbar_init(&idxbar[0], 1);
        mbar_init(&idxbar[1], 1);
        *abort_word = 0;
        *issued_word = 0;
        *idx_issued = 0;
        *idx_waited = 0;
        last_word[0] = last_word[1] = -1;
        fence_mbar_init();
    }
    __syncthreads();

    if (warp >= ncw) {
        // ---------------- producer warps ----------------
        // warp ncw issues the bulk copies and the index lists; every
        // producer warp gathers its share of each tile's halo records
        constexpr int kChunks = kRec / 16;
        const bool lead = warp == ncw && lane == 0;
        const int pl = threadIdx.x - ncw * 32;  // lane among the producer warps
        // halo indices of tile j go to ring entry j & 1 (lists are padded to
        // a multiple of 4 entries, so each copy is a multiple of 16 bytes)
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
        if (lead && blockIdx.x < ntiles) issue_idx(0, ti);
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
                if (ok && lead) *idx_waited = k + 1;
            }
            // a consumer group that gave up raised the abort word: no copy is
            // issued after that, so the drain below waits only for copies
            // that are certain to complete (the producer warps decide as one)
            if (group_any(kProdBar, kProdThreads, !ok || *abort_word)) {
                if (lead) {
                    *abort_word = 1;
                    atomicOr(a.err, 1);
                }
                break;
            }
            uint8_t *st = smem + (int64_t)s * L.stage;
            if (lead) {
                tinfo[s] = ti;  // published by the arrival below
                fence_proxy_async();
                const uint32_t eb = (uint32_t)ti.ne * kSlot, ab = (uint32_t)ti.nact * kSlot;
                const uint32_t ib = (uint32_t)ti.inc_words * 2u, sb = (uint32_t)ti.nm * kRec;
                mbar_expect_tx(&full[s], eb + ab + ib + sb);
                // read once per step: evict first from L2
                const uint64_t pol = l2_evict_first_policy();
                issue_chunks_hint(st + L.slots,
                                  reinterpret_cast<const uint8_t *>(a.ent) + (int64_t)ti.ent_off * kSlot, eb, &full[s],
                                  pol);
                issue_chunks_hint(st + L.act, reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * kSlot,
                                  ab, &full[s], pol);
                issue_chunks_hint(st + L.inc, reinterpret_cast<const uint8_t *>(a.inc + ti.inc_off), ib, &full[s], pol);
            }
            // slab, actuation, incidence and halo-index blocks are constant
            // across steps; the state records are the previous step's output
            if (k == 0) grid_dep_wait();
            if (lead) issue_chunks(st, in + (int64_t)ti.mass_off * kRec, (uint32_t)ti.nm * kRec, &full[s]);
            // halo records, one per producer lane at a time (their issue is
            // on the critical path)
            const int32_t *ix = idxbuf + (k & 1) * L.idx_words;
            for (int h = pl; h < ti.nh; h += kProdThreads) {
                const uint8_t *src = in + (int64_t)ix[h] * kRec;
                uint8_t *dst = st + (int64_t)(ti.nm + h) * kRec;
#pragma unroll
                for (int c = 0; c < kChunks; c++) cp_async16(dst + 16 * c, src + 16 * c);
            }
            cp_async_arrive(&full[s]);
            group_sync(kProdBar, kProdThreads);  // every producer lane has read ring entry k & 1
            if (lead) {
                *issued_word = k + 1;
                if (has_next) issue_idx(k + 1, tn);
            }
            ti = tn;
        }
    } else {
        // ---------------- consumer groups ----------------
        grid_dep_wait();  // the time record is the previous step's output
        const StepTime tm = step_time(a.tbuf[parity]);
        if (threadIdx.x == 0 && blockIdx.x == 0) a.tbuf[parity ^ 1] = tm.T + a.prm->launch_dt;
        const int grp = warp / gw;
        const int gt = threadIdx.x - grp * gw * 32;  // thread index within the group
        const int gn = gw * 32;
        const int bar_id = 1 + grp;
        R *sH = reinterpret_cast<R *>(smem + L.heavy) + grp * 3 * L.heavy_cap;
        for (int k = grp, t = blockIdx.x + grp * G; t < ntiles; k += 2, t += 2 * G) {
            const int s = k % NS;
            const uint32_t ph = (uint32_t)(k / NS) & 1u;
            const bool ok = bounded_wait(&full[s], ph, abort_word);
            if (group_any(bar_id, gn, !ok)) {
                if (gt == 0) {
                    *abort_word = 1;
                    atomicOr(a.err, 1);
                }
                break;
            }
            if (gt == 0) last_word[grp] = k;
            const TileInfo ti = tinfo[s];
            const int E = ti.ne;
            // per-mass scalars of this group's first masses (needed in phase
            // C; their loads overlap phase B)
            const int i_own = gt;
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
            uint8_t *st = smem + (int64_t)s * L.stage;
            uint8_t *slots = st + L.slots;
            const uint8_t *actb = st + L.act;
            const uint16_t *incs = reinterpret_cast<const uint16_t *>(st + L.inc);

            // ---- B: one force per slab entry, written over its record ----
            for (int e0 = gt; e0 < E; e0 += kBatchB * gn) {
                Rec16<PREC> r[kBatchB], q[kBatchB];
#pragma unroll
                for (int j = 0; j < kBatchB; j++) {
                    const int e = e0 + j * gn;
                    if (e < E) r[j] = load_rec<PREC>(slots + (int64_t)e * kSlot);
                    if (e < ti.nact) q[j] = load_rec<PREC>(actb + (int64_t)e * kSlot);
                }
#pragma unroll
                for (int j = 0; j < kBatchB; j++) {
                    const int e = e0 + j * gn;
                    if (e < E) entry_force<PREC>(r[j], e < ti.nact, q[j], st, tm, slots + (int64_t)e * kSlot);
                }
            }
            // the zero force that padding codes name (slot E)
            if (gt == 0) {
                reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[0] = make_float4(0.f, 0.f, 0.f, 0.f);
                if constexpr (kSlot == 32)
                    reinterpret_cast<float4 *>(slots + (int64_t)E * kSlot)[1] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            group_sync(bar_id, gn);

            // ---- C0: heavy masses ----
            if (ti.nheavy > 0) {
                heavy_sums<PREC>(a, ti, slots, sH, warp - grp * gw, gw);
                group_sync(bar_id, gn);
            }

            // ---- C: per-mass gather, constraints, integration ----
            for (int i = gt; i < ti.nm; i += gn) {
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
                    const uint32_t woff =
                        (own ? woff_own : __ldg(a.warp_inc_off + ti.warp_off + (i >> 5))) - (uint32_t)ti.inc_off;
                    const uint2 *ip = reinterpret_cast<const uint2 *>(incs + woff) + (i & 31);
                    const uint32_t nw = (d + 3) >> 2;
                    for (uint32_t w = 0; w < nw; w++) gather_word_padded<PREC>(slots, ip[32 * w], F0, F1, F2);
                }
                St<PREC> sv = load_state_smem<PREC>(st, i);
                integrate<PREC, INTEG>(a, ti, g, fl, m, F0, F1, F2, sv, out, g, write_acc, np, prm);
            }
            // the stage is free once every warp of the group is past it; order
            // this thread's slot writes before the copies that will reuse it
            fence_proxy_async();
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[s]);
        }
    }

    // drain: copies issued for tiles nobody consumed and index lists nobody
    // waited for (only after an abort)
    __syncthreads();
    if (threadIdx.x == 0) {
        const int issued = *issued_word;
        for (int k = 0; k < issued; k++) {
            if (k <= last_word[k & 1]) continue;
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
const void *ws_kernel(int integ) {
    switch (integ) {
        case INTEG_VERLET: return (const void *)k_step_ws<PREC, INTEG_VERLET>;
        case INTEG_RK2: return (const void *)k_step_ws<PREC, INTEG_RK2>;
        default: return (const void *)k_step_ws<PREC, INTEG_EULER>;
    }
}

const void *ws_kernel(int precision, int integ) {
    return precision == P_FP64   ? ws_kernel<P_FP64>(integ)
           : precision == P_FP32 ? ws_kernel<P_FP32>(integ)
                                 : ws_kernel<P_FP32C>(integ);
}

}  // namespace

cudaError_t step_ws_prepare(int precision, int integ, size_t smem) {
    return raise_smem_limit(ws_kernel(precision, integ), smem);
}

cudaError_t launch_step_ws(int precision, int integ, const StepArgs &a, int ctas, int consumer_warps, int parity,
                           int write_acc, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (consumer_warps < 2 || consumer_warps > kWsMaxConsumerWarps || (consumer_warps & 1))
        return cudaErrorInvalidValue;
    // programmatic stream serialisation: the next step's grid may start
    // while this one drains (the kernel orders its dependent reads itself)
    void *args[] = {const_cast<StepArgs *>(&a), &parity, &write_acc};
    return launch_programmatic(ws_kernel(precision, integ), dim3(ctas), dim3((consumer_warps + kWsProducerWarps) * 32), args,
                               (size_t)a.ws.total, s);
}

}  // namespace tg
