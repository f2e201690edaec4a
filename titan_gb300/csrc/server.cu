// server.cu -- device-resident request loop: many independent scenes
// (rollout requests) stepped by one persistent kernel.
//
// The reference runs one scene per process, on a host thread that launches
// two kernels per step and synchronises after each (src/sim.cu:1389-1428,
// 1503-1617).  Here one cooperative, persistent kernel (one 256-thread CTA
// per SM) holds a table of slots, each a started scene (its StepArgs: plan,
// records and state buffers, all already on the device) with a number of
// steps to go.  It loops over steps:
//   * boundary (CTA 0): slots whose steps are done retire -- the slot's
//     ticket is written to page-locked host memory, which the host polls --
//     and new requests are admitted from a ring the host writes in
//     page-locked memory (slot indices; the slot record itself was copied
//     to the device before the ring entry was published), then the step's
//     work list is built: the tiles of every active slot, as prefix sums;
//   * work (all CTAs): the work items, statically strided over the grid,
//     each one tile of one slot stepped by the whole CTA with the per-tile
//     kernel's phases (tile_step: the same arithmetic and order, so a
//     scene's result is bit-identical to its step() run and does not depend
//     on the other scenes);
//   * grid barriers (bounded) separate the phases.
// Data that other CTAs, CTA 0 or the host wrote during the kernel's life
// (state and time records, slot records, the work list) is read around L1
// (__ldcg): an SM's L1 may still hold an older copy.
// Every wait is bounded by the GPU clock: a barrier that is not reached in
// kBarrierNs, or host memory that stays silent past kIdleNs with no active
// slot, ends the kernel with a status word the host reads; the host
// relaunches it when it has work again.  A host-set stop word ends it at the
// next step boundary.  Euler steps only; two 256-thread CTAs per SM with
// the per-tile kernel's register-capped code (80 registers), so that other
// kernels (the scenes' transfers) keep room on each SM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.h"
#include "step_kernel.cuh"
#include "titan_gb300.h"

namespace tg {

namespace {

constexpr int kServeThreads = 256;
constexpr size_t kServeTileSmem = 112000;  // default shared memory for one tile
constexpr int kServeCtasPerSm = 2;  // 2 x 256 threads x 96 registers leaves a quarter of the file
constexpr int kRing = 16384;                     // ring entries (>= max slots)
constexpr uint64_t kBarrierNs = 20000000000ull;  // 20 s
constexpr uint64_t kIdleNs = 1000000000ull;      // 1 s without work: leave (the host relaunches)

enum { SS_RUNNING = 1, SS_STOPPED = 2, SS_IDLE = 3, SS_TIMEOUT = 4 };

// A slot: one scene and its remaining steps (device memory).
struct ServeSlot {
    StepArgs args;
    int64_t steps_left;
    uint64_t ticket;
    int32_t parity, ntiles;
    int32_t stepped;  // stepped in the last work phase
    int32_t pad;
};

// Control words and the per-step work list (device memory).
struct ServeCtl {
    unsigned bar_count, bar_gen;
    int exit_flag, nactive, total, pad0;
    uint64_t tail;  // ring entries admitted
};

// Page-locked host memory, mapped into the device.
struct ServeHost {
    uint64_t head;    // ring entries published by the host
    uint64_t tail;    // ring entries admitted (written by the kernel)
    int32_t stop;     // set by the host: leave at the next boundary
    int32_t status;   // SS_* (written by the kernel)
    int32_t ring[kRing];
    // followed by uint64_t done[max_slots]: the ticket of each slot's last finished request
};

__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint64_t ld_sys_u64(const uint64_t *p) {
    uint64_t v;
    asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_sys_s32(const int32_t *p) {
    int v;
    asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_sys_u64(uint64_t *p, uint64_t v) {
    asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_sys_s32(int32_t *p, int v) {
    asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier (the grid is co-resident: cooperative launch).  Bounded:
// false when it was not reached within kBarrierNs (the caller leaves).
__device__ bool grid_sync(ServeCtl *ctl) {
    __syncthreads();
    __shared__ int ok;
    if (threadIdx.x == 0) {
        volatile unsigned *gen = &ctl->bar_gen;
        const unsigned g = *gen;
        __threadfence();
        ok = 1;
        if (atomicAdd(&ctl->bar_count, 1u) == gridDim.x - 1) {
            atomicExch(&ctl->bar_count, 0u);
            __threadfence();
            atomicAdd(&ctl->bar_gen, 1u);
        } else {
            const uint64_t t0 = now_ns();
            while (*gen == g) {
                if (now_ns() - t0 > kBarrierNs) {
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// CTA 0 at a step boundary: finish the last step's bookkeeping, retire
// finished slots (ticket to the host), admit new ones from the ring, build
// the work list.  Sets ctl->exit_flag (and host->status) to leave.
__device__ void boundary(ServeSlot *slots, ServeCtl *ctl, int *active, int *prefix, int *scratch, ServeHost *host,
                         uint64_t *done, int max_slots) {
    __shared__ int s_n, s_exit;
    const int tid = threadIdx.x;
    if (tid == 0) s_n = __ldcg(&ctl->nactive);
    __syncthreads();
    const int n = s_n;
    // the last step: advance parity and count, mark the finished
    for (int j = tid; j < n; j += blockDim.x) {
        ServeSlot &sl = slots[__ldcg(active + j)];
        int64_t left = __ldcg(&sl.steps_left);
        if (__ldcg(&sl.stepped)) {
            sl.parity = __ldcg(&sl.parity) ^ 1;
            sl.steps_left = --left;
            sl.stepped = 0;
        }
        scratch[j] = left > 0;
    }
    __syncthreads();
    if (tid == 0) {
        // every CTA's writes of the finished slots are visible device-wide
        // (grid barrier); make them visible before the host hears of them
        __threadfence_system();
        int m = 0;
        for (int j = 0; j < n; j++) {
            const int si = __ldcg(active + j);
            if (scratch[j])
                active[m++] = si;
            else
                st_sys_u64(done + si, __ldcg(&slots[si].ticket));
        }
        // admit: ring entries published since the last admission (the host
        // never publishes more than its free slots)
        uint64_t tail = __ldcg(&ctl->tail);
        int exit_now = 0;
        const uint64_t t_idle = now_ns();
        for (;;) {
            const uint64_t head = ld_sys_u64(&host->head);
            while (tail < head && m < max_slots) {
                const int si = ld_sys_s32(host->ring + (tail % kRing));
                tail++;
                if (si >= 0 && si < max_slots && __ldcg(&slots[si].steps_left) > 0) active[m++] = si;
            }
            if (ld_sys_s32(&host->stop)) {
                exit_now = SS_STOPPED;
                break;
            }
            if (m > 0) break;
            if (now_ns() - t_idle > kIdleNs) {
                exit_now = SS_IDLE;
                break;
            }
            __nanosleep(2000);
        }
        ctl->tail = tail;
        st_sys_u64(&host->tail, tail);
        ctl->nactive = m;
        s_n = m;
        s_exit = exit_now;
        if (exit_now) {
            ctl->exit_flag = 1;
            st_sys_s32(&host->status, exit_now);
        }
    }
    __syncthreads();
    if (s_exit) return;
    // prefix sums of the active slots' tiles: each thread a chunk, then the
    // chunk totals scanned by thread 0
    const int m = s_n;
    const int per = (m + blockDim.x - 1) / blockDim.x;
    const int j0 = min(m, tid * per), j1 = min(m, j0 + per);
    int sum = 0;
    for (int j = j0; j < j1; j++) sum += __ldcg(&slots[__ldcg(active + j)].ntiles);
    scratch[tid] = sum;
    __syncthreads();
    if (tid == 0) {
        int acc = 0;
        for (int q = 0; q < (int)blockDim.x; q++) {
            const int v = scratch[q];
            scratch[q] = acc;
            acc += v;
        }
        ctl->total = acc;
        prefix[m] = acc;
    }
    __syncthreads();
    int acc = scratch[tid];
    for (int j = j0; j < j1; j++) {
        prefix[j] = acc;
        acc += __ldcg(&slots[__ldcg(active + j)].ntiles);
    }
}

// 96 registers a thread (80, the cap for three CTAs per SM, spilled 134
// bytes; 96: 0.275 against 0.307 ms per 100^3 step): two CTAs then hold
// three quarters of the register file, and the scenes' transfer kernels
// (256 threads of about 32 registers) still run beside the loop.
template <int PREC>
__global__ void __maxnreg__(96)
    k_serve(ServeSlot *slots, ServeCtl *ctl, int *active, int *prefix, int *scratch, ServeHost *host,
            uint64_t *done, int max_slots) {
    extern __shared__ __align__(16) uint8_t smem[];
    StepArgs *sa = reinterpret_cast<StepArgs *>(smem);
    uint8_t *tile_smem = smem + ((sizeof(StepArgs) + 15) & ~size_t(15));
    __shared__ int s_slot, s_local, s_parity, s_last;
    if (blockIdx.x == 0 && threadIdx.x == 0) st_sys_s32(&host->status, SS_RUNNING);
    bool timed_out = false;
    for (;;) {
        if (blockIdx.x == 0) boundary(slots, ctl, active, prefix, scratch, host, done, max_slots);
        if (!grid_sync(ctl)) {
            timed_out = true;
            break;
        }
        if (__ldcg(&ctl->exit_flag)) break;
        const int total = __ldcg(&ctl->total), n = __ldcg(&ctl->nactive);
        for (int w = blockIdx.x; w < total; w += gridDim.x) {
            if (threadIdx.x == 0) {
                int lo = 0, hi = n;  // the last j with prefix[j] <= w
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (__ldcg(prefix + mid) <= w)
                        lo = mid;
                    else
                        hi = mid;
                }
                const int si = __ldcg(active + lo);
                s_slot = si;
                s_local = w - __ldcg(prefix + lo);
                s_parity = __ldcg(&slots[si].parity);
                s_last = __ldcg(&slots[si].steps_left) == 1;
            }
            __syncthreads();
            const int *src = reinterpret_cast<const int *>(&slots[s_slot].args);
            for (int q = threadIdx.x; q < (int)(sizeof(StepArgs) / 4); q += blockDim.x)
                reinterpret_cast<int *>(sa)[q] = __ldcg(src + q);
            __syncthreads();
            const int local = s_local;
            const TileInfo ti = sa->tiles[local];
            // the per-tile kernel's register-capped configuration (LBM 3: two
            // slab entries in flight, no incidence prefetch)
            tile_step<PREC, 3, INTEG_EULER, true>(*sa, ti, tile_smem, s_parity, s_last, local == 0);
            __syncthreads();
        }
        if (!grid_sync(ctl)) {
            timed_out = true;
            break;
        }
        // every active slot was stepped once (all its tiles done)
        if (blockIdx.x == 0)
            for (int j = threadIdx.x; j < n; j += blockDim.x) slots[__ldcg(active + j)].stepped = 1;
    }
    if (timed_out && threadIdx.x == 0) st_sys_s32(&host->status, SS_TIMEOUT);
}

const void *serve_kernel(int prec) {
    return prec == P_FP64   ? (const void *)k_serve<P_FP64>
           : prec == P_FP32 ? (const void *)k_serve<P_FP32>
                            : (const void *)k_serve<P_FP32C>;
}

}  // namespace
}  // namespace tg

using tg::ServeCtl;
using tg::ServeHost;
using tg::ServeSlot;

struct titan_gb300_server {
    int device = 0, prec = 0, max_slots = 0, ctas = 0;
    size_t smem = 0, tile_smem = 0;
    cudaStream_t run_stream = nullptr, ctl_stream = nullptr;
    ServeSlot *d_slots = nullptr;
    ServeCtl *d_ctl = nullptr;
    int *d_active = nullptr, *d_prefix = nullptr, *d_scratch = nullptr;
    ServeHost *h_host = nullptr;  // page-locked, mapped
    uint64_t *h_done = nullptr;   // inside h_host's allocation
    ServeHost *d_host = nullptr;  // its device address
    uint64_t *d_done = nullptr;
    std::mutex mu;
    std::vector<int> free_slots;
    struct Req {
        titan_gb300_sim *sim = nullptr;
        int64_t nsteps = 0;
        uint64_t ticket = 0;
    };
    std::vector<Req> req;  // per slot
    std::unordered_map<uint64_t, int> slot_of;  // ticket -> slot, requests in flight
    uint64_t next_ticket = 0;
    int64_t launches = 0;
    bool launched = false;
    std::string err;
    int fail(int code, const std::string &m) {
        err = m;
        return code;
    }
};

namespace {

int srv_cuda(titan_gb300_server *s, cudaError_t e, const char *what) {
    return s->fail(TITAN_GB300_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Launches the kernel when it is not running and the host has published
// requests it has not admitted (it leaves after kIdleNs without work, and
// may have left just before a publication).
int ensure_running(titan_gb300_server *s) {
    if (s->launched) {
        const cudaError_t q = cudaStreamQuery(s->run_stream);
        if (q == cudaErrorNotReady) return TITAN_GB300_OK;
        if (q != cudaSuccess) return srv_cuda(s, q, "server kernel");
        s->launched = false;
        if (__atomic_load_n(&s->h_host->status, __ATOMIC_ACQUIRE) == tg::SS_TIMEOUT)
            return s->fail(TITAN_GB300_ETIMEOUT, "the server kernel's bounded grid barrier gave up");
    }
    const uint64_t head = __atomic_load_n(&s->h_host->head, __ATOMIC_ACQUIRE);
    const uint64_t tail = __atomic_load_n(&s->h_host->tail, __ATOMIC_ACQUIRE);
    if (head == tail) return TITAN_GB300_OK;
    s->h_host->status = 0;
    cudaError_t e = cudaMemsetAsync(&s->d_ctl->exit_flag, 0, sizeof(int), s->run_stream);
    if (e != cudaSuccess) return srv_cuda(s, e, "server launch");
    void *args[] = {&s->d_slots, &s->d_ctl, &s->d_active, &s->d_prefix, &s->d_scratch, &s->d_host, &s->d_done,
                    &s->max_slots};
    e = cudaLaunchCooperativeKernel(tg::serve_kernel(s->prec), dim3(s->ctas), dim3(tg::kServeThreads), args, s->smem,
                                    s->run_stream);
    if (e != cudaSuccess) return srv_cuda(s, e, "server launch");
    s->launched = true;
    s->launches++;
    return TITAN_GB300_OK;
}

}  // namespace

extern "C" {

int titan_gb300_server_create(titan_gb300_server **out, int device, int precision, int max_slots,
                              int64_t tile_smem_bytes) try {
    if (!out) return TITAN_GB300_EINVAL;
    *out = nullptr;
    if (precision < 0 || precision > 2 || max_slots < 1 || max_slots > tg::kRing || tile_smem_bytes < 0)
        return TITAN_GB300_EINVAL;
    auto *s = new (std::nothrow) titan_gb300_server();
    if (!s) return TITAN_GB300_ENOMEM;
    // every failure below releases what was made so far
    auto bail = [s](int code) {
        titan_gb300_server_destroy(s);
        return code;
    };
    s->device = device;
    s->prec = precision;
    s->max_slots = max_slots;
    // default: room for a 208-mass FP32C tile of a lattice (about 103 KB of
    // records) while two CTAs, each with its launch parameters, still share
    // one SM (2 x 112,352 bytes)
    s->tile_smem = tile_smem_bytes > 0 ? (size_t)tile_smem_bytes : tg::kServeTileSmem;
    s->smem = ((sizeof(tg::StepArgs) + 15) & ~size_t(15)) + s->tile_smem;
    if (cudaSetDevice(device) != cudaSuccess) return bail(TITAN_GB300_ECUDA);
    const void *f = tg::serve_kernel(precision);
    if (tg::raise_smem_limit(f, s->smem) != cudaSuccess) return bail(TITAN_GB300_ELIMIT);
    int sms = 0, per_sm = 0, coop = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (!coop || sms < 1) return bail(TITAN_GB300_ECUDA);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, f, tg::kServeThreads, s->smem) != cudaSuccess ||
        per_sm < 1)
        return bail(TITAN_GB300_ELIMIT);
    // two CTAs per SM where they fit: the register cap and the tile budget
    // leave each SM room for other kernels (the scenes' transfers)
    s->ctas = sms * std::min(per_sm, tg::kServeCtasPerSm);
    if (cudaStreamCreateWithFlags(&s->run_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->ctl_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(TITAN_GB300_ECUDA);
    if (cudaMalloc(&s->d_slots, sizeof(ServeSlot) * max_slots) != cudaSuccess ||
        cudaMalloc(&s->d_ctl, sizeof(ServeCtl)) != cudaSuccess ||
        cudaMalloc(&s->d_active, sizeof(int) * max_slots) != cudaSuccess ||
        cudaMalloc(&s->d_prefix, sizeof(int) * (max_slots + 1)) != cudaSuccess ||
        cudaMalloc(&s->d_scratch, sizeof(int) * std::max(max_slots, tg::kServeThreads)) != cudaSuccess)
        return bail(TITAN_GB300_ENOMEM);
    if (cudaMemset(s->d_slots, 0, sizeof(ServeSlot) * max_slots) != cudaSuccess ||
        cudaMemset(s->d_ctl, 0, sizeof(ServeCtl)) != cudaSuccess)
        return bail(TITAN_GB300_ECUDA);
    const size_t hb = sizeof(ServeHost) + sizeof(uint64_t) * max_slots;
    void *h = nullptr;
    if (cudaHostAlloc(&h, hb, cudaHostAllocMapped) != cudaSuccess) return bail(TITAN_GB300_ENOMEM);
    std::memset(h, 0, hb);
    s->h_host = static_cast<ServeHost *>(h);
    s->h_done = reinterpret_cast<uint64_t *>(static_cast<uint8_t *>(h) + sizeof(ServeHost));
    if (cudaHostGetDevicePointer((void **)&s->d_host, h, 0) != cudaSuccess) return bail(TITAN_GB300_ECUDA);
    s->d_done = reinterpret_cast<uint64_t *>(reinterpret_cast<uint8_t *>(s->d_host) + sizeof(ServeHost));
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(TITAN_GB300_ECUDA);
    s->req.assign(max_slots, {});
    for (int i = max_slots - 1; i >= 0; i--) s->free_slots.push_back(i);
    *out = s;
    return TITAN_GB300_OK;
} catch (...) {
    return TITAN_GB300_ENOMEM;
}

int titan_gb300_server_submit(titan_gb300_server *s, titan_gb300_sim *sim, int64_t nsteps, int64_t *ticket) try {
    if (!s || !sim || !ticket || nsteps < 1) return TITAN_GB300_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->free_slots.empty()) return s->fail(TITAN_GB300_EBUSY, "no free slot");
    tg::ServeScene v{};
    std::string why;
    const int rc = tg::serve_begin(sim, s->device, s->prec, s->tile_smem, v, why);
    if (rc) return s->fail(rc, why);
    if (cudaSetDevice(s->device) != cudaSuccess) {
        tg::serve_end(sim, 0);
        return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    }
    const int si = s->free_slots.back();
    ServeSlot sl{};
    sl.args = *v.args;
    sl.steps_left = nsteps;
    sl.ticket = ++s->next_ticket;
    sl.parity = v.parity;
    sl.ntiles = v.args->ntiles;
    cudaError_t e = cudaMemcpyAsync(s->d_slots + si, &sl, sizeof(sl), cudaMemcpyHostToDevice, s->ctl_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctl_stream);
    if (e != cudaSuccess) {
        tg::serve_end(sim, 0);
        return srv_cuda(s, e, "submit");
    }
    s->free_slots.pop_back();
    s->req[si] = {sim, nsteps, sl.ticket};
    s->slot_of[sl.ticket] = si;
    const uint64_t head = s->h_host->head;
    s->h_host->ring[head % tg::kRing] = si;
    __atomic_store_n(&s->h_host->head, head + 1, __ATOMIC_RELEASE);
    *ticket = (int64_t)sl.ticket;
    return ensure_running(s);
} catch (...) {
    return TITAN_GB300_ENOMEM;
}

int titan_gb300_server_poll(titan_gb300_server *s, int64_t ticket) try {
    if (!s || ticket < 1) return TITAN_GB300_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    const auto it = s->slot_of.find((uint64_t)ticket);
    if (it == s->slot_of.end()) return s->fail(TITAN_GB300_EINVAL, "no such request in flight");
    const int si = it->second;
    if (__atomic_load_n(s->h_done + si, __ATOMIC_ACQUIRE) == (uint64_t)ticket) {
        tg::serve_end(s->req[si].sim, s->req[si].nsteps);
        s->req[si] = {};
        s->slot_of.erase(it);
        s->free_slots.push_back(si);
        return TITAN_GB300_OK;
    }
    const int rc = ensure_running(s);
    return rc ? rc : TITAN_GB300_EBUSY;
} catch (...) {
    return TITAN_GB300_ENOMEM;
}

int titan_gb300_server_info(const titan_gb300_server *s, int64_t out[6]) {
    if (!s || !out) return TITAN_GB300_EINVAL;
    out[0] = s->max_slots - (int64_t)s->free_slots.size();
    out[1] = (int64_t)s->free_slots.size();
    out[2] = s->launches;
    out[3] = s->h_host ? __atomic_load_n(&s->h_host->status, __ATOMIC_ACQUIRE) : 0;
    out[4] = s->ctas;
    out[5] = (int64_t)s->smem;
    return TITAN_GB300_OK;
}

const char *titan_gb300_server_last_error(const titan_gb300_server *s) { return s ? s->err.c_str() : "null handle"; }

void titan_gb300_server_destroy(titan_gb300_server *s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->h_host) __atomic_store_n(&s->h_host->stop, 1, __ATOMIC_RELEASE);
    if (s->run_stream) cudaStreamSynchronize(s->run_stream);
    for (auto &r : s->req)
        if (r.sim) tg::serve_end(r.sim, -1);  // unfinished: the scene keeps what its last step left
    if (s->d_slots) cudaFree(s->d_slots);
    if (s->d_ctl) cudaFree(s->d_ctl);
    if (s->d_active) cudaFree(s->d_active);
    if (s->d_prefix) cudaFree(s->d_prefix);
    if (s->d_scratch) cudaFree(s->d_scratch);
    if (s->h_host) cudaFreeHost(s->h_host);
    if (s->run_stream) cudaStreamDestroy(s->run_stream);
    if (s->ctl_stream) cudaStreamDestroy(s->ctl_stream);
    delete s;
}

}  // extern "C"
