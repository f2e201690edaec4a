// step_tma.cu -- pipelined persistent form of the fused step (sm_103a).
//
// Same arithmetic, same per-mass summation order and same results as k_step
// (step.cu) -- the tests check the two bit for bit -- but organised so that
// HBM traffic overlaps computation:
//   * a persistent grid (a few CTAs per SM) walks the tiles;
//   * while a CTA computes tile k, the Tensor Memory Accelerator streams
//     tile k+1's slab records, actuation records, incidence block and tile
//     state records into the other shared-memory stage (cp.async.bulk with
//     an mbarrier transaction count), and the CTA's threads fetch tile k+1's
//     halo state records with 16-byte cp.async;
//   * the halo index list of tile k+2 rides in tile k+1's bulk group, so the
//     halo gathers can be issued a full tile ahead;
//   * each entry's force overwrites its consumed record in shared memory, and
//     the per-mass gather reads it back as one 16-byte vector.
// Every mbarrier wait is bounded: on time-out the kernel sets *err, drains
// its own copies (bounded) and returns; the host reports the error.
#include <cstdint>

#include "async_copy.cuh"
#include "engine.h"
#include "epilogue.cuh"
#include "state.cuh"
#include "step_math.cuh"
#include "tile_phases.cuh"

namespace tg {

namespace {

template <int PREC>
struct Geo {
    static constexpr int kRec = PREC == P_FP32 ? 32 : 48;  // state record bytes
    static constexpr int kEnt = PREC == P_FP64 ? 32 : 16;  // slab / actuation record bytes
};

template <int PREC>
__device__ __forceinline__ void issue_tile(const StepArgs &a, const TileInfo &ti, const void *in, uint8_t *stage,
                                           const TileInfo *ti2, uint8_t *idxbuf, uint64_t *bar) {
    using G = Geo<PREC>;
    const PipeLayout &L = a.pipe;
    uint32_t bytes = (uint32_t)ti.ne * G::kEnt + (uint32_t)ti.nact * G::kEnt + (uint32_t)ti.inc_words * 2 +
                     (uint32_t)ti.nm * G::kRec;
    uint32_t nh2 = ti2 ? (uint32_t)((ti2->nh + 3) & ~3) : 0u;
    bytes += nh2 * 4;
    mbar_expect_tx(bar, bytes);
    const uint8_t *ent = reinterpret_cast<const uint8_t *>(a.ent) + (int64_t)ti.ent_off * G::kEnt;
    const uint8_t *act = reinterpret_cast<const uint8_t *>(a.act) + (int64_t)ti.ent_off * G::kEnt;
    issue_chunks(stage + L.rec, ent, (uint32_t)ti.ne * G::kEnt, bar);
    issue_chunks(stage + L.act, act, (uint32_t)ti.nact * G::kEnt, bar);
    issue_chunks(stage + L.inc, reinterpret_cast<const uint8_t *>(a.inc + ti.inc_off), (uint32_t)ti.inc_words * 2,
                 bar);
    issue_chunks(stage + L.st, reinterpret_cast<const uint8_t *>(in) + (int64_t)ti.mass_off * G::kRec,
                 (uint32_t)ti.nm * G::kRec, bar);
    if (nh2) issue_chunks(idxbuf, reinterpret_cast<const uint8_t *>(a.halo + ti2->halo_off), nh2 * 4, bar);
}

// Halo state records of tile ti into stage (after its tile masses).
template <int PREC>
__device__ __forceinline__ void issue_halo(const TileInfo &ti, const void *in, uint8_t *st, const int32_t *idx) {
    using G = Geo<PREC>;
    constexpr int kChunks = G::kRec / 16;
    const int n = ti.nh * kChunks;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int h = q / kChunks, c = q - h * kChunks;
        const uint8_t *src = reinterpret_cast<const uint8_t *>(in) + (int64_t)idx[h] * G::kRec + 16 * c;
        cp_async16(st + (int64_t)(ti.nm + h) * G::kRec + 16 * c, src);
    }
}

// Bounded wait on a stage's mbarrier; false (and *err set) on time-out.
__device__ __forceinline__ bool wait_stage(const StepArgs &a, uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < kWaitLimit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(a.err, 1);
    return false;
}

template <int PREC>
__global__ void __launch_bounds__(512) k_step_pipe(StepArgs a, int parity, int write_acc) {
    using R = typename Real<PREC>::T;
    using G = Geo<PREC>;
    extern __shared__ __align__(128) uint8_t smem[];
    const PipeLayout &L = a.pipe;
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.mbar);
    R *sH = reinterpret_cast<R *>(smem + L.heavy);
    const void *in = parity ? a.state1 : a.state0;
    void *out = parity ? a.state0 : a.state1;
    const int64_t np = a.npad;
    const DevParams *prm = a.prm;
    const StepTime tm = step_time(a.tbuf[parity]);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.tbuf[parity ^ 1] = tm.T + prm->launch_dt;
    const int ntiles = a.ntiles;
    const int t0 = blockIdx.x;
    if (t0 >= ntiles) return;
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    // this CTA's tile descriptors (tiles t0, t0+G, ...), cached so that no
    // iteration waits on a global load before issuing its copies
    TileInfo *tcache = reinterpret_cast<TileInfo *>(smem + L.tinfo);
    {
        const int words = (int)(sizeof(TileInfo) / 4);
        for (int q = threadIdx.x; q < kPipeTileCache * words; q += blockDim.x) {
            const int k = q / words, w = q - k * words;
            const int t = blockIdx.x + k * (int)gridDim.x;
            if (t < ntiles)
                reinterpret_cast<int32_t *>(tcache + k)[w] = __ldg(reinterpret_cast<const int32_t *>(a.tiles + t) + w);
        }
    }
    auto tile = [&](int k) -> TileInfo {
        return k < kPipeTileCache ? tcache[k] : a.tiles[blockIdx.x + k * (int)gridDim.x];
    };
    __syncthreads();

    // Pipeline invariant: at the start of iteration k (tile t0 + kG, stage
    // k & 1), index buffer (k+1) & 1 holds the halo indices of tile
    // t0 + (k+1)G.  Prologue: tile t0 (with its own halo indices in buffer 0)
    // into stage 0, its halo gathers, and the indices of t0 + G into buffer 1.
    uint32_t phase[2] = {0u, 0u};
    const int G_ = gridDim.x;
    const TileInfo first = tile(0);
    if (threadIdx.x == 0) issue_tile<PREC>(a, first, in, smem, &first, smem + L.idx, &bars[0]);
    // every wait outcome is made block-uniform before anyone acts on it
    bool ok = !__syncthreads_or(!wait_stage(a, &bars[0], 0));
    phase[0] ^= 1u;
    if (ok) issue_halo<PREC>(first, in, smem + L.st, reinterpret_cast<const int32_t *>(smem + L.idx));
    cp_async_commit();
    if (t0 + G_ < ntiles) {
        const TileInfo ti1 = tile(1);
        int32_t *idx1 = reinterpret_cast<int32_t *>(smem + L.idx + L.idx_bytes);
        for (int h = threadIdx.x; h < ti1.nh; h += blockDim.x) idx1[h] = __ldg(a.halo + ti1.halo_off + h);
    }
    __syncthreads();

    int k = 0;
    for (int t = t0; t < ntiles && ok; t += G_, k++) {
        const int s = k & 1;
        uint8_t *stage = smem + s * L.stage;
        uint8_t *next_stage = smem + (s ^ 1) * L.stage;
        const TileInfo ti = tile(k);
        const int tn = t + G_;
        const bool has_next = tn < ntiles;
        TileInfo tin{};
        if (has_next) tin = tile(k + 1);
        // (a) bulk copies of tile t+G (and the halo indices of t+2G) into the other stage
        if (threadIdx.x == 0 && has_next) {
            const int tnn = tn + G_;
            TileInfo tinn{};
            if (tnn < ntiles) tinn = tile(k + 2);
            fence_proxy_async();
            issue_tile<PREC>(a, tin, in, next_stage, tnn < ntiles ? &tinn : nullptr,
                             smem + L.idx + s * L.idx_bytes, &bars[s ^ 1]);
        }
        // per-mass scalars of this tile, needed only in phase C
        const int i_own = threadIdx.x;
        uint8_t fl = MF_FIXED;
        uint32_t dg = 0, woff = 0;
        R m = 1;
        if (i_own < ti.nm) {
            const int64_t g = (int64_t)ti.mass_off + i_own;
            fl = __ldg(a.flags + g);
            dg = __ldg(a.deg + g);
            m = __ldg(reinterpret_cast<const R *>(a.mass) + g);
            woff = __ldg(a.warp_inc_off + ti.warp_off + (i_own >> 5)) - (uint32_t)ti.inc_off;
        }
        // (b) this tile's bulk data
        if (k > 0) {
            const bool timed_out = !wait_stage(a, &bars[s], phase[s]);
            if (!timed_out) phase[s] ^= 1u;
            if (__syncthreads_or(timed_out)) {
                ok = false;
                break;
            }
        }
        // (c) halo gathers of the next tile (its indices are in buffer s^1)
        if (has_next)
            issue_halo<PREC>(tin, in, next_stage + L.st,
                             reinterpret_cast<const int32_t *>(smem + L.idx + (s ^ 1) * L.idx_bytes));
        cp_async_commit();
        // (d) this tile's halo gathers (committed one group earlier)
        cp_async_wait_1();
        __syncthreads();

        const uint8_t *st = stage + L.st;
        uint8_t *recb = stage + L.rec;
        const uint8_t *actb = stage + L.act;
        const uint16_t *incs = reinterpret_cast<const uint16_t *>(stage + L.inc);

        // ---- B: one force per slab entry, written over its record --------
        for (int e = threadIdx.x; e < ti.ne; e += blockDim.x) {
            uint8_t *slot = recb + (int64_t)e * G::kEnt;
            const bool actuated = e < ti.nact;
            const Rec16<PREC> r = load_rec<PREC>(slot);
            const Rec16<PREC> q = actuated ? load_rec<PREC>(actb + (int64_t)e * G::kEnt) : r;
            entry_force<PREC>(r, actuated, q, st, tm, slot);
        }
        __syncthreads();

        // ---- C0: heavy masses (warp-cooperative, fixed order) --------------
        if (ti.nheavy > 0) {
            heavy_sums<PREC>(a, ti, recb, sH, threadIdx.x >> 5, blockDim.x >> 5);
            __syncthreads();
        }

        // ---- C: per-mass gather, constraints, integration ------------------
        for (int i = threadIdx.x; i < ti.nm; i += blockDim.x) {
            const int64_t g = (int64_t)ti.mass_off + i;
            uint8_t fli = fl;
            uint32_t d = dg, wo = woff;
            R mi = m;
            if (i != i_own) {  // more masses than threads
                fli = __ldg(a.flags + g);
                d = __ldg(a.deg + g);
                mi = __ldg(reinterpret_cast<const R *>(a.mass) + g);
                wo = __ldg(a.warp_inc_off + ti.warp_off + (i >> 5)) - (uint32_t)ti.inc_off;
            }
            if (fli & MF_FIXED) continue;
            R F0 = 0, F1 = 0, F2 = 0;
            if (d == 255) {
                int h = 0;
                while (h < ti.nheavy && a.heavy_local[ti.heavy_off + h] != i) h++;
                F0 = F0 + sH[h];
                F1 = F1 + sH[ti.nheavy + h];
                F2 = F2 + sH[2 * ti.nheavy + h];
            } else {
                const uint2 *ip = reinterpret_cast<const uint2 *>(incs + wo) + (i & 31);
                const uint32_t nw = (d + 3) >> 2;
                for (uint32_t w = 0; w < nw; w++) gather_word<PREC>(recb, ip[32 * w], w, d, F0, F1, F2);
            }
            St<PREC> sv = load_state_smem<PREC>(st, i);
            integrate<PREC>(a, ti, g, fli, mi, F0, F1, F2, sv, out, g, write_acc, np, prm);
        }
        __syncthreads();  // the stage and the index buffer are free again
    }
    if (!ok) {
        // drain this CTA's own copies before returning (bounded)
        cp_async_wait_all();
        for (int s = 0; s < 2; s++) {
            uint32_t it = 0;
            while (it++ < kWaitLimit && !mbar_try_wait(&bars[s], phase[s])) {
            }
        }
    } else {
        cp_async_wait_all();
    }
}

}  // namespace

int state_record_bytes(int precision) { return precision == P_FP32 ? 32 : 48; }
int entry_record_bytes(int precision) { return precision == P_FP64 ? 32 : 16; }

cudaError_t step_pipe_prepare(int precision, size_t smem) {
    const void *f = precision == P_FP64   ? (const void *)k_step_pipe<P_FP64>
                    : precision == P_FP32 ? (const void *)k_step_pipe<P_FP32>
                                          : (const void *)k_step_pipe<P_FP32C>;
    return raise_smem_limit(f, smem);
}

cudaError_t launch_step_pipe(int precision, const StepArgs &a, int ctas, int threads, int parity, int write_acc,
                             cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    const size_t smem = (size_t)a.pipe.total;
    switch (precision) {
        case P_FP64: k_step_pipe<P_FP64><<<ctas, threads, smem, s>>>(a, parity, write_acc); break;
        case P_FP32: k_step_pipe<P_FP32><<<ctas, threads, smem, s>>>(a, parity, write_acc); break;
        default: k_step_pipe<P_FP32C><<<ctas, threads, smem, s>>>(a, parity, write_acc); break;
    }
    return cudaGetLastError();
}

}  // namespace tg
