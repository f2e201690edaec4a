// capi.cu -- the C ABI of include/titan_gb300.h.
//
// Replaces the reference's device-state layer and run loop
// (src/sim.cu:821-1017 AoS per-object cudaMalloc + pointer arrays, and
// src/sim.cu:1503-1617 sync + two launches per step) with: one tile plan,
// structure-of-arrays buffers allocated once, and CUDA-graph replay of the
// fused step kernel on a private stream.
#include "titan_gb300.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <chrono>
#include <cstring>
#include <thread>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "engine.h"
#include "plan.h"

using tg::P_FP32;
using tg::P_FP32C;
using tg::P_FP64;

namespace {

constexpr int kChunk = 64;  // steps per cached graph

double norm3(const double *v) {
    double a = v[0] * v[0], b = v[1] * v[1], c = v[2] * v[2];
    return std::sqrt((a + b) + c);
}

struct DevMem {
    std::vector<void *> ptrs;
    size_t total = 0;
    void *get(size_t bytes, cudaError_t &e) {
        void *p = nullptr;
        if (bytes == 0) bytes = 16;
        e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) {
            ptrs.push_back(p);
            total += bytes;
        }
        return p;
    }
    void release() {
        for (void *p : ptrs) cudaFree(p);
        ptrs.clear();
        total = 0;
    }
};

}  // namespace

struct titan_gb300_sim {
    int device = 0, prec = P_FP64;
    cudaStream_t stream = nullptr;
    // resident tiles run on side_stream beside the per-step kernels
    cudaStream_t side_stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string err;

    // host scene (creation order)
    int64_t n = 0;
    std::vector<double> pos, vel, m, ext, drag_in;
    std::vector<uint8_t> fixed;
    std::vector<int32_t> drag;
    std::vector<int64_t> lc_ptr;  // n+1 or empty
    std::vector<int32_t> lc_type;
    std::vector<double> lc_rec;   // 4 per record
    int64_t ns = 0;
    std::vector<int32_t> left, right, type;
    std::vector<double> k, rest, damping, omega, amp, phase;
    std::vector<std::array<double, 6>> planes;
    std::vector<std::array<double, 4>> balls;
    std::vector<int64_t> body_ptr;
    std::vector<std::array<double, 6>> body_plane;
    std::vector<uint8_t> body_has_plane;
    double dt = 1e-4;
    double g[3] = {0.0, 0.0, -9.81};

    // run state
    bool started = false;
    double T = 0.0;
    int64_t steps = 0;
    int parity = 0;
    std::vector<double> mT0;       // per-mass local time at its last upload
    std::vector<int64_t> mTstep;   // step count at that upload
    struct DtSeg {
        int64_t first;  // first step of the segment
        double dt;
        int halves;     // 2: RK2 advances time by dt/2 twice per step
    };
    std::vector<DtSeg> dt_log;
    int integrator = tg::INTEG_EULER;
    int passes() const { return integrator == tg::INTEG_RK2 ? 2 : 1; }

    // device
    tg::Plan plan;
    DevMem mem;
    tg::StepArgs args{};
    tg::DevParams hprm{};
    tg::DevParams *dprm = nullptr;
    int threads = 512;
    int tile_masses = 0;
    size_t smem = 0;
    int64_t npad = 0;
    int32_t *d_old2new = nullptr;
    double *d_xfer = nullptr;     // 9n doubles
    int64_t *d_idx = nullptr;     // n
    double *h_xfer = nullptr;     // pinned 9n doubles
    std::map<std::pair<int, int>, cudaGraphExec_t> graphs;
    // diagnostics (lazy)
    int32_t *d_sl = nullptr, *d_sr = nullptr;
    double *d_sk = nullptr, *d_srest = nullptr, *d_partials = nullptr, *d_dout = nullptr;

    size_t rsize() const { return prec == P_FP64 ? sizeof(double) : sizeof(float); }
    int comps() const { return tg::state_words(prec); }
    int threads_req = 0;  // CTA size override (0: derived from the tile size)
    int min_ctas_req = 0; // register cap of the per-tile kernel: 0/1 none, 3 or 4 CTAs per SM
    int step_variant = 0; // launch-bound variant in use (engine.h)
    int kernel_req = 0;   // 0 auto, 1 per-tile kernel, 3 per-tile with async staging, 4 warp-specialised, 6 pull
    bool use_async = false;
    bool use_ws = false;
    bool serving = false;  // handed to a request server (server.cu)
    bool use_pull = false;
    tg::PullTables pull;  // host copy of the pull form's spring tables
    std::vector<tg::PullTile> pull_tiles;
    int64_t pull_impl_bytes = 0;
    int ws_warps = 0;     // consumer warps of the warp-specialised kernel
    int ctas = 0;         // persistent grid of the pipelined kernel
    int *d_err = nullptr;
    // body-resident batched launch
    int res_mode = -1;    // -1 automatic, 0 off, 1 bins of whole bodies, 2 halo-free tiles
    int res_bin_req = 0;  // bin capacity in masses (0: default)
    int res_threads_req = 0;
    tg::ResPlan rplan;
    tg::ResArgs rargs{};
    bool use_res = false;
    int res_threads = 0, res_ctas = 0;
    // resident tiles (mode 2): halo-free tiles stepped in shared memory
    bool use_rtiles = false;
    tg::TileResArgs rtargs{};
    std::vector<tg::TileInfo> rtiles;
    int rt_threads = 0, rt_mpt = 0;
    size_t rt_smem = 0;
    // plan taken from another handle with the same topology (adopt_plan);
    // used by the first start() only
    bool plan_adopted = false;
    int plan_tile = 0;  // tile size the current plan was built with
    int plan_req = 0;   // tile size requested for it (0: the default)

    cudaError_t launch(int parity, int write_acc, int stage = 0) {
        if (args.ntiles == 0) return cudaSuccess;
        args.rk2_stage = stage;
        if (use_pull) return tg::launch_step_pull(prec, integrator, args, ctas, parity, write_acc, stream);
        if (use_ws) return tg::launch_step_ws(prec, integrator, args, ctas, ws_warps, parity, write_acc, stream);
        if (use_async)
            return tg::launch_step_async(prec, args, (int)args.ntiles, threads, smem, parity, write_acc, stream);
        return tg::launch_step(prec, step_variant, integrator, args, (int)args.ntiles, threads, smem, parity,
                               write_acc, stream);
    }

    int fail(int code, const std::string &msg) {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return TITAN_GB300_ECUDA;
    }

    void drop_graphs() {
        for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
        graphs.clear();
    }
    void free_device() {
        drop_graphs();
        mem.release();
        if (h_xfer) cudaFreeHost(h_xfer);
        h_xfer = nullptr;
        d_sl = d_sr = nullptr;
        d_sk = d_srest = d_partials = d_dout = nullptr;
    }
    ~titan_gb300_sim() {
        if (stream) cudaStreamSynchronize(stream);
        free_device();
        if (stream) cudaStreamDestroy(stream);
        if (side_stream) {
            cudaStreamSynchronize(side_stream);
            cudaStreamDestroy(side_stream);
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
    }
};

namespace {

#define CK(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return s->cuda_fail(e_, what); \
    } while (0)

// Whether a caller's host buffer is page-locked (cudaMallocHost or
// cudaHostRegister): such buffers are copied by DMA directly, without the
// staging copy through the handle's own pinned buffer.
bool host_pinned(const void *p) {
    if (!p) return false;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // clear the error state the failed query left
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// memcpy of large host buffers split over a few threads (the staging copies
// of whole-scene state are tens of MB; one core copies them at a fraction of
// the host memory bandwidth).
void par_memcpy(void *dst, const void *src, size_t bytes) {
    constexpr size_t kPiece = 8u << 20;
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = std::min<size_t>(std::min<size_t>(8, hw), (bytes + kPiece - 1) / kPiece);
    if (nt <= 1) {
        std::memcpy(dst, src, bytes);
        return;
    }
    const size_t per = (bytes / nt + 63) & ~size_t(63);
    std::vector<std::thread> th;
    for (size_t q = 1; q < nt; q++) {
        const size_t o = q * per;
        if (o >= bytes) break;
        th.emplace_back([=] {
            std::memcpy(static_cast<uint8_t *>(dst) + o, static_cast<const uint8_t *>(src) + o, std::min(per, bytes - o));
        });
    }
    std::memcpy(dst, src, std::min(per, bytes));
    for (auto &t : th) t.join();
}

uint8_t mass_flags(const titan_gb300_sim *s, int64_t i) {
    uint8_t f = 0;
    if (!s->fixed.empty() && s->fixed[i]) f |= tg::MF_FIXED;
    if (!s->ext.empty() && (s->ext[3 * i] != 0.0 || s->ext[3 * i + 1] != 0.0 || s->ext[3 * i + 2] != 0.0))
        f |= tg::MF_EXT;
    if (!s->drag.empty() && s->drag[i] != 0) f |= tg::MF_DRAG;
    if (!s->lc_ptr.empty() && s->lc_ptr[i + 1] > s->lc_ptr[i]) f |= tg::MF_LOCAL;
    return f;
}

void fill_params(titan_gb300_sim *s) {
    tg::DevParams &p = s->hprm;
    std::memset(&p, 0, sizeof(p));
    p.dt = s->dt;
    p.dt_hi = (float)s->dt;
    p.dt_lo = (float)(s->dt - (double)p.dt_hi);
    p.integrator = s->integrator;
    p.dt2 = std::pow(s->dt, 2);
    p.dt2f = (float)p.dt2;
    p.launch_dt = s->integrator == tg::INTEG_RK2 ? 0.5 * s->dt : s->dt;
    for (int c = 0; c < 3; c++) {
        p.g[c] = s->g[c];
        p.gf[c] = (float)s->g[c];
    }
    p.nplanes = (int32_t)s->planes.size();
    p.nballs = (int32_t)s->balls.size();
    for (size_t j = 0; j < s->planes.size(); j++)
        for (int c = 0; c < 6; c++) {
            p.plane[j][c] = s->planes[j][c];
            p.planef[j][c] = (float)s->planes[j][c];
        }
    for (size_t j = 0; j < s->balls.size(); j++)
        for (int c = 0; c < 4; c++) {
            p.ball[j][c] = s->balls[j][c];
            p.ballf[j][c] = (float)s->balls[j][c];
        }
}

int upload_params(titan_gb300_sim *s) {
    fill_params(s);
    CK(cudaMemcpyAsync(s->dprm, &s->hprm, sizeof(tg::DevParams), cudaMemcpyHostToDevice, s->stream),
       "upload params");
    CK(cudaMemcpyAsync(s->args.tbuf + s->parity, &s->T, sizeof(double), cudaMemcpyHostToDevice, s->stream),
       "upload time");
    CK(cudaStreamSynchronize(s->stream), "upload params");
    return TITAN_GB300_OK;
}

template <typename R>
std::vector<R> to_real(const std::vector<double> &v) {
    return std::vector<R>(v.begin(), v.end());
}

// Per-mass device arrays (m, flags, ext, drag, local constraints) from the
// host mirror, in tiled order.
int upload_mass_attrs(titan_gb300_sim *s) {
    const tg::Plan &P = s->plan;
    const int64_t n = s->n, np = s->npad;
    std::vector<uint8_t> flags(np, tg::MF_FIXED);
    std::vector<double> md(np, 1.0), extd(3 * np, 0.0);
    std::vector<int32_t> dragn(np, 0), lcp(np + 1, 0);
    std::vector<int32_t> lct;
    std::vector<double> lcr;
    for (int64_t g = 0; g < n; g++) {
        int64_t i = P.new2old[g];
        uint8_t f = mass_flags(s, i);
        int32_t b = 0;
        if (!s->body_ptr.empty())
            b = (int32_t)(std::upper_bound(s->body_ptr.begin(), s->body_ptr.end(), i) - s->body_ptr.begin() - 1);
        if (!s->body_has_plane.empty() && s->body_has_plane[b]) f |= tg::MF_BODYPLANE;
        flags[g] = f;
        md[g] = s->m[i];
        if (!s->ext.empty())
            for (int c = 0; c < 3; c++) extd[c * np + g] = s->ext[3 * i + c];
        if (!s->drag.empty()) dragn[g] = s->drag[i];
        lcp[g] = (int32_t)lct.size();
        if (!s->lc_ptr.empty())
            for (int64_t r = s->lc_ptr[i]; r < s->lc_ptr[i + 1]; r++) {
                lct.push_back(s->lc_type[r]);
                for (int c = 0; c < 4; c++) lcr.push_back(s->lc_rec[4 * r + c]);
            }
    }
    for (int64_t g = n; g <= np; g++) lcp[g] = (int32_t)lct.size();
    auto &a = s->args;
    CK(cudaMemcpy(const_cast<uint8_t *>(a.flags), flags.data(), np, cudaMemcpyHostToDevice), "upload flags");
    if (s->prec == P_FP64) {
        CK(cudaMemcpy(const_cast<void *>(a.mass), md.data(), np * 8, cudaMemcpyHostToDevice), "upload m");
        CK(cudaMemcpy(const_cast<void *>(a.ext), extd.data(), 3 * np * 8, cudaMemcpyHostToDevice), "upload ext");
    } else {
        auto mf = to_real<float>(md);
        auto ef = to_real<float>(extd);
        CK(cudaMemcpy(const_cast<void *>(a.mass), mf.data(), np * 4, cudaMemcpyHostToDevice), "upload m");
        CK(cudaMemcpy(const_cast<void *>(a.ext), ef.data(), 3 * np * 4, cudaMemcpyHostToDevice), "upload ext");
    }
    CK(cudaMemcpy(const_cast<int32_t *>(a.drag), dragn.data(), np * 4, cudaMemcpyHostToDevice), "upload drag");
    CK(cudaMemcpy(const_cast<int32_t *>(a.lc_ptr), lcp.data(), (np + 1) * 4, cudaMemcpyHostToDevice), "upload lc");
    if (!lct.empty()) {
        cudaError_t e;
        int32_t *t = (int32_t *)s->mem.get(lct.size() * 4, e);
        if (!t) return s->cuda_fail(e, "alloc lc");
        double *r = (double *)s->mem.get(lcr.size() * 8, e);
        if (!r) return s->cuda_fail(e, "alloc lc");
        CK(cudaMemcpy(t, lct.data(), lct.size() * 4, cudaMemcpyHostToDevice), "upload lc");
        CK(cudaMemcpy(r, lcr.data(), lcr.size() * 8, cudaMemcpyHostToDevice), "upload lc");
        a.lc_type = t;
        a.lc_rec = r;
    }
    return TITAN_GB300_OK;
}

tg::PullSprings pull_springs(const titan_gb300_sim *s) {
    tg::PullSprings sp;
    sp.k = s->k.data();
    sp.rest = s->rest.data();
    sp.damping = s->damping.empty() ? nullptr : s->damping.data();
    return sp;
}

// Spring records (slab-entry layout: FP64 k, rest, damping, word; FP32
// word, k, rest, damping) and actuation records for the springs spring[e]
// with entry words word[e] (spring -1: a zero padding record), uploaded to
// rec / act.
int upload_records(titan_gb300_sim *s, const std::vector<int64_t> &spring, const std::vector<uint32_t> &word,
                   void *rec, void *act) {
    const size_t E = spring.size();
    if (E == 0) return TITAN_GB300_OK;
    auto sp_amp = [&](int64_t j) { return s->amp.empty() ? 0.2 : s->amp[j]; };
    auto sp_phase = [&](int64_t j) { return s->phase.empty() ? 0.0 : s->phase[j]; };
    auto sp_omega = [&](int64_t j) { return s->omega.empty() ? 0.0 : s->omega[j]; };
    if (s->prec == P_FP64) {
        std::vector<double> ent(4 * E, 0.0), ac(4 * E, 0.0);
        for (size_t e = 0; e < E; e++) {
            int64_t j = spring[e];
            if (j < 0) continue;
            ent[4 * e] = s->k[j];
            ent[4 * e + 1] = s->rest[j];
            ent[4 * e + 2] = s->damping[j];
            uint64_t bits = word[e];
            std::memcpy(&ent[4 * e + 3], &bits, 8);
            ac[4 * e] = sp_omega(j);
            ac[4 * e + 1] = sp_amp(j);
            ac[4 * e + 2] = sp_phase(j);
        }
        CK(cudaMemcpy(rec, ent.data(), ent.size() * 8, cudaMemcpyHostToDevice), "upload records");
        CK(cudaMemcpy(act, ac.data(), ac.size() * 8, cudaMemcpyHostToDevice), "upload actuation");
    } else {
        std::vector<float> ent(4 * E, 0.f), ac(4 * E, 0.f);
        for (size_t e = 0; e < E; e++) {
            int64_t j = spring[e];
            if (j < 0) continue;
            uint32_t bits = word[e];
            std::memcpy(&ent[4 * e], &bits, 4);
            ent[4 * e + 1] = (float)s->k[j];
            ent[4 * e + 2] = (float)s->rest[j];
            ent[4 * e + 3] = (float)s->damping[j];
            // rest' = rest (1 + a sin(2 pi (nu T + phi))): nu = omega / 2 pi,
            // phi = phase / 2 pi, a = -amp for contract-then-expand (type 2)
            const double two_pi = 6.283185307179586476925286766559;
            const int ty = s->type.empty() ? 0 : s->type[j];
            ac[4 * e] = (float)(sp_omega(j) / two_pi);
            ac[4 * e + 1] = (float)(ty == 2 ? -sp_amp(j) : sp_amp(j));
            ac[4 * e + 2] = (float)(sp_phase(j) / two_pi);
            ac[4 * e + 3] = (float)s->rest[j];  // read by the pull form with the record
        }
        CK(cudaMemcpy(rec, ent.data(), ent.size() * 4, cudaMemcpyHostToDevice), "upload records");
        CK(cudaMemcpy(act, ac.data(), ac.size() * 4, cudaMemcpyHostToDevice), "upload actuation");
    }
    return TITAN_GB300_OK;
}

// Slab entry records and actuation parameters from the host spring arrays,
// and the resident bins' records.
int upload_entries(titan_gb300_sim *s) {
    const tg::Plan &P = s->plan;
    auto &a = s->args;
    int rc = upload_records(s, P.ent_spring, P.ent_ends, const_cast<void *>(a.ent), const_cast<void *>(a.act));
    if (rc) return rc;
    if (s->use_pull && a.pull_units) {  // new spring parameters: same layout, new values
        tg::PullTables T;
        std::string why = tg::build_pull(P, s->pull_tiles, s->pull.team_warps, tg::state_record_bytes(s->prec) / 16,
                                         pull_springs(s), T);
        if (!why.empty()) return s->fail(TITAN_GB300_ELIMIT, why);
        if (T.units.size() != s->pull.units.size() || T.ell.size() != s->pull.ell.size())
            return s->fail(TITAN_GB300_EINVAL, "pull tables changed shape without a new plan");
        s->pull = std::move(T);
        CK(cudaMemcpy(const_cast<tg::PullUnit *>(a.pull_units), s->pull.units.data(),
                      s->pull.units.size() * sizeof(tg::PullUnit), cudaMemcpyHostToDevice),
           "upload pull units");
        CK(cudaMemcpy(const_cast<uint8_t *>(a.pull_ell), s->pull.ell.data(), s->pull.ell.size(),
                      cudaMemcpyHostToDevice),
           "upload pull columns");
    }
    if (s->use_res)
        rc = upload_records(s, s->rplan.rec_spring, s->rplan.words, const_cast<void *>(s->rargs.rec),
                            const_cast<void *>(s->rargs.act));
    return rc;
}

template <typename T>
T *dev_copy(titan_gb300_sim *s, const std::vector<T> &v, cudaError_t &e) {
    T *p = (T *)s->mem.get(v.size() * sizeof(T), e);
    if (!p) return nullptr;
    if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? p : nullptr;
}

// default tile of the warp-specialised form, and its fallback when two
// stages of the default's tiles do not fit one SM's shared memory
constexpr int kWsDefaultTile = 208;
constexpr int kWsFallbackTile = 192;
// default tile of the pull form: seven 32-mass units, one per warp of a team
// (two teams and the producer: 16 warps, four per SM sub-partition)
constexpr int kPullDefaultTile = 224;
// the automatic kernel choice in FP32 and FP32C: the warp-specialised form
// (measured faster on GB300 on the 100^3 lattice: 0.121 ms per step against
// 0.134 for the pull form with 160-mass tiles and three teams)
constexpr bool kPullAuto = false;
constexpr int kHeavyThreshold = 96;

// Whether the step will run the pull form: when requested (set_kernel 6).
// (It needs a plan without heavy masses: it has no warp-cooperative sums.)
bool pull_wanted(const titan_gb300_sim *s) {
    if (s->kernel_req == 6) return true;
    if (!kPullAuto || s->kernel_req != 0 || s->prec == P_FP64) return false;
    std::vector<int32_t> deg(s->n, 0);
    for (int64_t j = 0; j < s->ns; j++) {
        const int64_t l = s->left[j], r = s->right[j];
        if (l < 0 || r < 0 || l >= s->n || r >= s->n) continue;
        if (++deg[l] > kHeavyThreshold && (s->fixed.empty() || !s->fixed[l])) return false;
        if (++deg[r] > kHeavyThreshold && (s->fixed.empty() || !s->fixed[r])) return false;
    }
    return true;
}

tg::PlanInput plan_input(titan_gb300_sim *s, int tile_masses) {
    tg::PlanInput in;
    in.n = s->n;
    in.pos = s->pos.data();
    in.fixed = s->fixed.empty() ? nullptr : s->fixed.data();
    in.ns = s->ns;
    in.left = s->left.data();
    in.right = s->right.data();
    in.type = s->type.empty() ? nullptr : s->type.data();
    in.nbodies = s->body_ptr.empty() ? 0 : (int64_t)s->body_ptr.size() - 1;
    in.body_ptr = s->body_ptr.empty() ? nullptr : s->body_ptr.data();
    // Default tile.  Large scenes: 256 masses in FP64 (with two threads per
    // mass: the FP64 pipe wants the warps; 2.40 ms per 100^3 step against
    // 2.50 with tiles of 128), 208 for the FP32 forms' warp-specialised
    // kernel (two stages fit one SM's shared memory; 192 where they would
    // not, plan_scene) and 256 for the per-tile forms.  Smaller scenes get
    // smaller tiles so that their tiles cover the SMs: FP64 about 1.6 tiles
    // per SM (tiles of 32 to 256 masses), the warp-specialised form about
    // 4 (64 to 208).  In the FP32 forms a body that fits the large-scene
    // tile stays whole (a halo-free tile runs resident: 2.0 us per step for
    // the 5^3 lattice against 3.3 split in four); in FP64, bound by each
    // SM's FP64 pipe, it is split like the rest (17.9 us in four tiles
    // against 28.9 resident).  Measured on GB300, 20^3 lattice: FP64 37 us
    // per step with 32-mass tiles against 90 with 256; FP32C 5.3 us with
    // 64 against 6.5 with 208.
    const bool pull = pull_wanted(s);
    const bool ws = !pull && (s->kernel_req == 0 || s->kernel_req == 4);
    if (tile_masses > 0) {
        in.tile_cap = tile_masses;
    } else {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device) != cudaSuccess || sms <= 0) {
            cudaGetLastError();
            sms = 152;  // GB300
        }
        auto fit = [&](double per_sm, int lo, int hi) {
            const int64_t t = (int64_t)((double)s->n / (per_sm * sms)) / 32 * 32;
            return (int)std::max<int64_t>(lo, std::min<int64_t>(hi, t));
        };
        if (s->prec == P_FP64) {
            in.tile_cap = fit(1.6, 32, 256);  // small bodies split too: FP64 binds per SM
        } else if (pull) {
            in.tile_cap = fit(4.0, 64, kPullDefaultTile);
            in.whole_cap = kPullDefaultTile;
        } else if (ws) {
            in.tile_cap = fit(4.0, 64, kWsDefaultTile);
            in.whole_cap = kWsDefaultTile;
        } else {
            in.tile_cap = 256;
        }
    }
    in.heavy_threshold = kHeavyThreshold;
    // a tile's staged state, entry forces and heavy sums share one CTA's
    // shared memory (tile_smem_bytes)
    const int rs = (int)s->rsize();
    in.slot_cap = 4095;
    in.entry_cap = 32767;
    in.smem_budget = 220 * 1024;
    in.slot_bytes = tg::state_record_bytes(s->prec);
    in.entry_bytes = tg::entry_record_bytes(s->prec);
    in.heavy_bytes = 3 * rs;
    return in;
}

// Bin capacity of the resident plan (0: no resident bins): two state
// records per mass must fit one CTA's shared memory, with at most
// kResMaxMpt masses per thread.
int resident_cap(const titan_gb300_sim *s) {
    const int64_t nb = s->body_ptr.empty() ? 1 : (int64_t)s->body_ptr.size() - 1;
    const bool want = s->res_mode == 1;
    if (!want) return 0;
    const int rec = tg::state_record_bytes(s->prec);
    int lim = (int)(((227 * 1024 - 1024) / (2 * rec)) & ~31);
    lim = std::min(lim, tg::kResMaxMpt * (s->res_threads_req > 0 ? s->res_threads_req : 512));
    int64_t big = 0, fit = 0;
    for (int64_t b = 0; b < nb; b++) {
        const int64_t m = s->body_ptr.empty() ? s->n : s->body_ptr[b + 1] - s->body_ptr[b];
        if (m <= lim) big = std::max(big, m), fit++;
    }
    if (big == 0) return 0;
    // default: bins of at least 1024 masses pack small bodies; with no more
    // bodies than one wave of single-body bins (152 SMs), one body per bin
    // of its own size (more CTAs, less shared memory each)
    const int64_t dflt = fit <= 152 ? big : std::max<int64_t>(1024, big);
    const int cap = s->res_bin_req > 0 ? s->res_bin_req : (int)dflt;
    return std::min(lim, (cap + 31) & ~31);
}

// Per-tile launch records of a plan.
std::vector<tg::TileInfo> tile_infos(const tg::Plan &P) {
    std::vector<tg::TileInfo> tiles(P.ntiles);
    for (int64_t t = 0; t < P.ntiles; t++) {
        tg::TileInfo &ti = tiles[t];
        ti.mass_off = (int32_t)P.tile_mass_off[t];
        ti.nm = (int32_t)(P.tile_mass_off[t + 1] - P.tile_mass_off[t]);
        ti.halo_off = (int32_t)P.tile_halo_off[t];
        ti.nh = P.tile_nh[t];
        ti.ent_off = (int32_t)P.tile_ent_off[t];
        ti.ne = (int32_t)(P.tile_ent_off[t + 1] - P.tile_ent_off[t]);
        ti.nact = P.tile_nact[t];
        ti.warp_off = (int32_t)P.tile_warp_off[t];
        ti.heavy_off = (int32_t)P.tile_heavy_off[t];
        ti.nheavy = (int32_t)(P.tile_heavy_off[t + 1] - P.tile_heavy_off[t]);
        ti.body = P.body_of_tile[t];
        const int64_t w0 = P.tile_warp_off[t], w1 = P.tile_warp_off[t + 1];
        const int64_t i0 = w1 > w0 ? (int64_t)P.warp_inc_off[w0] : 0;
        const int64_t i1 = w1 > w0 ? (w1 < (int64_t)P.warp_inc_off.size() ? (int64_t)P.warp_inc_off[w1]
                                                                           : (int64_t)P.inc.size())
                                   : 0;
        ti.inc_off = (int32_t)i0;
        ti.inc_words = (int32_t)(i1 - i0);
        ti.pad0 = ti.pad1 = ti.pad2 = 0;
    }
    return tiles;
}

// Stage layout of the warp-specialised kernel for these tiles (sized by
// their largest): the offsets inside a stage, the halo-index and heavy-sum
// capacities, and how many stages fit one SM's shared memory (nstages; the
// kernel needs at least two).
void ws_stage_layout(int prec, const std::vector<tg::TileInfo> &tiles, tg::WsLayout &W) {
    auto al = [](int64_t x, int64_t q) { return (x + q - 1) / q * q; };
    const int rec = tg::state_record_bytes(prec), ent = tg::entry_record_bytes(prec);
    const int64_t rs = prec == P_FP64 ? 8 : 4;
    int64_t mS = 0, mE = 0, mH = 0, mNh = 0, mA = 0, mI = 0;
    for (const tg::TileInfo &ti : tiles) {
        mS = std::max<int64_t>(mS, ti.nm + ti.nh);
        mE = std::max<int64_t>(mE, ti.ne);
        mH = std::max<int64_t>(mH, ti.nheavy);
        mNh = std::max<int64_t>(mNh, ti.nh);
        mA = std::max<int64_t>(mA, ti.nact);
        mI = std::max<int64_t>(mI, ti.inc_words);
    }
    W.slots = (int32_t)al(mS * rec, 16);
    W.act = (int32_t)al(W.slots + (mE + 1) * ent, 16);  // + the zero slot padding codes name
    W.inc = (int32_t)al(W.act + mA * ent, 16);
    W.stage = (int32_t)al(W.inc + mI * 2, 128);
    W.idx_words = (int32_t)al(mNh, 4);
    W.heavy_cap = (int32_t)std::max<int64_t>(1, mH);
    const int64_t tail = 2 * (int64_t)W.idx_words * 4 + al(2 * 3 * (int64_t)W.heavy_cap * rs, 16) +
                         tg::kWsMaxStages * (int64_t)sizeof(tg::TileInfo) + al((int64_t)sizeof(tg::DevParams), 16) +
                         (2 * tg::kWsMaxStages + 2) * 8 + 32;
    const int64_t room = 227 * 1024 - tail;
    W.nstages = (int32_t)std::min<int64_t>(tg::kWsMaxStages, room / std::max<int64_t>(1, W.stage));
}

// Shared-memory layout of the pull kernel for these tiles (sized by their
// largest): stages of one tile's state records, as many as fit one SM (at
// most kPullMaxStages, a multiple of the team count, at least two per
// team).  Returns false when that many do not fit.
bool pull_layout(int prec, const std::vector<tg::TileInfo> &tiles, int threads_req, tg::PullLayout &L) {
    auto al = [](int64_t x, int64_t q) { return (x + q - 1) / q * q; };
    const int rec = tg::state_record_bytes(prec);
    int64_t mS = 0, mNm = 0, mNh = 0, mA = 0;
    for (const tg::TileInfo &ti : tiles) {
        mS = std::max<int64_t>(mS, ti.nm + ti.nh);
        mNm = std::max<int64_t>(mNm, ti.nm);
        mNh = std::max<int64_t>(mNh, ti.nh);
        mA = std::max<int64_t>(mA, ti.nact);
    }
    L = tg::PullLayout{};
    L.team_warps = (int32_t)std::max<int64_t>(1, (mNm + 31) / 32);
    if (L.team_warps > tg::kPullMaxConsumerWarps) return false;
    // two teams by default (one team's narrow tile start and end overlap
    // the other's streaming); set_launch's thread count asks for another
    const int want = threads_req > 0 ? threads_req / 32 / L.team_warps : 2;
    L.nteams = std::max(1, std::min(want, tg::kPullMaxConsumerWarps / L.team_warps));
    L.act_off = (int32_t)al(mS * rec, 16);
    L.stage = (int32_t)al(L.act_off + mA * 16, 128);
    L.idx_words = (int32_t)al(std::max<int64_t>(mNh, 1), 4);
    const int64_t tail = 2 * (int64_t)L.idx_words * 4 + al((int64_t)sizeof(tg::DevParams), 16) +
                         (2 * tg::kPullMaxStages + 2) * 8 + 32 + 32;
    const int64_t room = 227 * 1024 - tail;
    int64_t ns = std::min<int64_t>(tg::kPullMaxStages, room / std::max<int64_t>(1, L.stage));
    ns -= ns % L.nteams;
    if (ns < 2 * L.nteams) return false;
    L.nstages = (int32_t)ns;
    L.idx = (int32_t)(ns * L.stage);
    L.params = (int32_t)al(L.idx + 2 * (int64_t)L.idx_words * 4, 16);
    L.mbar = (int32_t)al(L.params + (int64_t)sizeof(tg::DevParams), 16);
    L.total = L.mbar + (2 * L.nstages + 2) * 8 + 32;
    return L.total <= 227 * 1024;
}

// Builds the pull form's tables and layout for the tiles the per-step
// kernel runs; on success sets use_pull.  A scene the pull form cannot run
// is an error only when it was requested.
int setup_pull(titan_gb300_sim *s, std::vector<tg::TileInfo> &tiles_run) {
    s->use_pull = false;
    if (s->prec == P_FP64) return s->fail(TITAN_GB300_EINVAL, "the pull kernel runs FP32 and FP32C only");
    std::vector<tg::PullTile> pt(tiles_run.size());
    for (size_t t = 0; t < tiles_run.size(); t++) {
        pt[t].mass_off = tiles_run[t].mass_off;
        pt[t].ent_off = tiles_run[t].ent_off;
        pt[t].warp_off = tiles_run[t].warp_off;
        pt[t].nm = tiles_run[t].nm;
    }
    tg::PullLayout L{};
    if (!pull_layout(s->prec, tiles_run, s->threads_req, L)) {
        if (s->kernel_req == 6) return s->fail(TITAN_GB300_ELIMIT, "two tiles per team do not fit the pull kernel's shared memory");
        return TITAN_GB300_OK;
    }
    std::string why = tg::build_pull(s->plan, pt, L.team_warps, tg::state_record_bytes(s->prec) / 16,
                                     pull_springs(s), s->pull);
    if (!why.empty()) {
        s->pull = tg::PullTables();
        if (s->kernel_req == 6) return s->fail(TITAN_GB300_ELIMIT, why);
        return TITAN_GB300_OK;
    }
    s->pull_tiles = std::move(pt);
    s->args.pull = L;
    // implementation bytes of one step: state records read (tile and halo)
    // and written, m and flags per mass, the spring quads of every unit
    // (damping quads included where they are read), the tiles' actuation
    // records, unit descriptors, halo indices and tile records
    const int64_t rec = tg::state_record_bytes(s->prec);
    int64_t nh = 0, nm = 0, nact = 0, quad_bytes = 0;
    for (const tg::TileInfo &ti : tiles_run) {
        nh += ti.nh;
        nm += ti.nm;
        nact += ti.nact;
    }
    for (const tg::PullUnit &pu : s->pull.units) quad_bytes += (int64_t)pu.nquads * tg::pull_quad_bytes(pu.flags & tg::PU_DAMP);
    s->pull_impl_bytes = nm * (2 * rec + 4 + 1) + nh * (rec + 4) + quad_bytes + nact * 16 +
                         (int64_t)s->pull.units.size() * 16 + (int64_t)tiles_run.size() * (int64_t)sizeof(tg::TileInfo);
    s->use_pull = true;
    return TITAN_GB300_OK;
}

// Builds s->plan for a requested tile size (0: the default).  The default
// tile of the warp-specialised form (208 masses) gives way to 192 when two
// stages of the planned tiles would not fit one SM's shared memory.
std::string plan_scene(titan_gb300_sim *s, int tile_masses, tg::PlanInput &in) {
    in = plan_input(s, tile_masses);
    std::string why = tg::build_plan(in, s->plan);
    if (why.empty() && tile_masses == 0 && in.tile_cap == kWsDefaultTile && !pull_wanted(s)) {
        tg::WsLayout W{};
        ws_stage_layout(s->prec, tile_infos(s->plan), W);
        if (W.nstages < 2) {
            in = plan_input(s, kWsFallbackTile);
            why = tg::build_plan(in, s->plan);
        }
    }
    s->plan_req = tile_masses;
    return why;
}

// Builds the plan and all device buffers; positions/velocities come from the
// host mirror.  Keeps T / steps.
int build_device(titan_gb300_sim *s) {
    s->free_device();
    tg::PlanInput in;
    const size_t rs = s->rsize();
    if (s->plan_adopted && !s->started && s->plan_req == s->tile_masses) {
        s->plan_adopted = false;  // the adopted plan serves this first start
        in = plan_input(s, s->plan_tile);
    } else {
        s->plan_adopted = false;
        std::string why = plan_scene(s, s->tile_masses, in);
        if (!why.empty()) return s->fail(TITAN_GB300_ELIMIT, why);
    }
    s->plan_tile = in.tile_cap;
    const tg::Plan &P = s->plan;
    // threads per CTA of the per-tile forms: one per tile mass (two in FP64)
    s->threads = s->threads_req > 0
                     ? s->threads_req
                     : std::max(128, std::min(512, ((P.max_nm + 31) / 32) * 32 * (s->prec == P_FP64 ? 2 : 1)));
    s->npad = ((s->n + 127) / 128) * 128;
    const int64_t np = s->npad;
    auto &a = s->args;
    a = tg::StepArgs{};
    a.npad = np;
    a.slots = std::max(P.max_slots, 1);
    a.ecap = std::max(P.max_entries, 1);
    a.hcap = std::max(P.max_heavy, 1);
    cudaError_t e = cudaSuccess;
    s->smem = 0;
    std::vector<tg::TileInfo> tiles = tile_infos(P);
    for (int64_t t = 0; t < P.ntiles; t++) {
        const tg::TileInfo &ti = tiles[t];
        // ne + 1 force slots: the last holds the zero force padding codes name
        s->smem = std::max(s->smem, s->kernel_req == 3
                                        ? tg::tile_async_smem_bytes(s->prec, ti.nm + ti.nh, ti.ne + 1, ti.nheavy)
                                        : tg::tile_smem_bytes(s->prec, ti.nm + ti.nh, ti.ne + 1, ti.nheavy));
    }
    if (P.inc.size() > (size_t)INT32_MAX) return s->fail(TITAN_GB300_ELIMIT, "incidence table exceeds 2^31 words");
    // body-resident bins: whole bodies that fit one CTA run all the steps of
    // a launch in shared memory; the per-step kernels take the other tiles
    s->use_res = false;
    s->rplan = tg::ResPlan();
    s->rargs = tg::ResArgs{};
    {
        const int cap = s->integrator == tg::INTEG_EULER ? resident_cap(s) : 0;
        if (cap > 0) {
            tg::build_resident(in, P, cap, cap, s->rplan);
            if (s->rplan.nbins > 0) {
                s->use_res = true;
                s->res_threads = s->res_threads_req > 0
                                     ? s->res_threads_req
                                     : std::max(128, std::min(512, ((cap + 1) / 2 + 31) & ~31));
                const int mpt = (cap + s->res_threads - 1) / s->res_threads;
                const size_t rsm = tg::resident_smem_bytes(s->prec, cap);
                CK(tg::resident_prepare(s->prec, mpt, rsm), "set resident shared memory");
                const int per_sm = tg::resident_ctas_per_sm(s->prec, mpt, s->res_threads, rsm);
                if (per_sm <= 0) return s->fail(TITAN_GB300_ELIMIT, "resident bins do not fit one SM");
                int sms = 0, dev = 0;
                CK(cudaGetDevice(&dev), "device");
                CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device");
                s->res_ctas = (int)std::min<int64_t>(s->rplan.nbins, (int64_t)sms * per_sm);
                s->rargs.nbins = s->rplan.nbins;
                s->rargs.cap = cap;
            }
        }
    }
    // resident tiles: halo-free tiles run all the steps of a launch in shared
    // memory, their slab, actuation and incidence records staged there too
    // when the largest tile's fit and every tile still gets a CTA at once
    s->use_rtiles = false;
    s->rtiles.clear();
    s->rtargs = tg::TileResArgs{};
    std::vector<uint8_t> rt_flag(P.ntiles, 0);
    // automatic: resident tiles for every halo-free tile that fits when the
    // kernel form is automatic (measured on GB300: 2.5x faster than the
    // per-step kernels on one 125-mass body, 2x on thousands of them, 5 %
    // on the 4096-body batch whose small bodies alone are halo-free;
    // never slower on the mixed scenes tried)
    const bool rt_auto = s->res_mode == -1 && s->kernel_req == 0;
    if ((s->res_mode == 2 || rt_auto) && s->integrator == tg::INTEG_EULER) {
        const size_t kMaxSmem = 227 * 1024;
        const int tcap = s->res_threads_req > 0 ? s->res_threads_req : 512;
        int64_t max_nm = 0, max_ne = 0;
        for (int64_t t = 0; t < P.ntiles; t++) {
            const tg::TileInfo &ti = tiles[t];
            if (ti.nh != 0 || ti.nm > tg::kResMaxMpt * tcap || tg::tile_resident_smem_bytes(s->prec, ti, 0) > kMaxSmem)
                continue;
            rt_flag[t] = 1;
            s->rtiles.push_back(ti);
            max_nm = std::max<int64_t>(max_nm, ti.nm);
            max_ne = std::max<int64_t>(max_ne, ti.ne);
        }
        if (!s->rtiles.empty()) {
            int sms = 0, dev = 0;
            CK(cudaGetDevice(&dev), "device");
            CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device");
            // threads: a thread per mass of the largest tile; with fewer tiles
            // than SMs, up to a quarter of its slab entries (phase B) -- in
            // [64, 512] (measured on GB300: one 125-mass tile steps fastest
            // with 288 threads, thousands of them with 128)
            const int64_t want_t = (int64_t)s->rtiles.size() < sms ? std::max<int64_t>(max_nm, max_ne / 4) : max_nm;
            s->rt_threads = s->res_threads_req > 0
                                ? s->res_threads_req
                                : (int)std::max<int64_t>(64, std::min<int64_t>(512, (want_t + 31) & ~int64_t(31)));
            s->rt_mpt = (int)((max_nm + s->rt_threads - 1) / s->rt_threads);
            size_t sm_st = 0, sm_pl = 0;
            for (const tg::TileInfo &ti : s->rtiles) {
                sm_st = std::max(sm_st, tg::tile_resident_smem_bytes(s->prec, ti, 1));
                sm_pl = std::max(sm_pl, tg::tile_resident_smem_bytes(s->prec, ti, 0));
            }
            int stage = 0;
            if (sm_st <= kMaxSmem && tg::tile_resident_prepare(s->prec, s->rt_mpt, 1, sm_st) == cudaSuccess) {
                const int ps = tg::tile_resident_ctas_per_sm(s->prec, s->rt_mpt, 1, s->rt_threads, sm_st);
                stage = ps > 0 && (int64_t)s->rtiles.size() <= (int64_t)sms * ps;
            }
            s->rt_smem = stage ? sm_st : sm_pl;
            CK(tg::tile_resident_prepare(s->prec, s->rt_mpt, stage, s->rt_smem), "set resident-tile shared memory");
            if (tg::tile_resident_ctas_per_sm(s->prec, s->rt_mpt, stage, s->rt_threads, s->rt_smem) <= 0)
                return s->fail(TITAN_GB300_ELIMIT, "resident tiles do not fit one SM");
            s->use_rtiles = true;
            s->rtargs.ntiles = (int32_t)s->rtiles.size();
            s->rtargs.stage = stage;
        }
    }
    std::vector<tg::TileInfo> tiles_run;
    for (int64_t t = 0; t < P.ntiles; t++)
        if ((!s->use_res || !s->rplan.tile_resident[t]) && !rt_flag[t]) tiles_run.push_back(tiles[t]);
    // automatic choice: the warp-specialised form in FP32 and FP32C (measured
    // fastest on GB300, see the kernel-form sweep in profiles/) when two of
    // the scene's tiles fit one SM's shared memory, else the per-tile form;
    // the per-tile form in FP64 (FP64-ALU bound, no gain from overlap)
    // the pull form when requested (or automatic, kPullAuto), else the
    // warp-specialised one
    s->use_pull = false;
    s->pull = tg::PullTables();
    s->pull_tiles.clear();
    if ((s->kernel_req == 6 || (kPullAuto && s->kernel_req == 0 && s->prec != P_FP64)) && !tiles_run.empty()) {
        int rc = setup_pull(s, tiles_run);
        if (rc) return rc;
    }
    s->use_ws = false;
    const bool want_ws =
        !s->use_pull && (s->kernel_req == 4 || (s->kernel_req == 0 && s->prec != P_FP64 && !tiles_run.empty()));
    if (want_ws) {
        tg::WsLayout &W = a.ws;
        ws_stage_layout(s->prec, tiles_run, W);
        if (W.nstages < 2 && s->kernel_req == 4)
            return s->fail(TITAN_GB300_ELIMIT, "two tiles do not fit in shared memory for the warp-specialised kernel");
    }
    if (want_ws && a.ws.nstages >= 2) {
        auto al = [](int64_t x, int64_t q) { return (x + q - 1) / q * q; };
        tg::WsLayout &W = a.ws;
        W.idx = W.nstages * W.stage;
        W.heavy = W.idx + 2 * W.idx_words * 4;
        W.tinfo = (int32_t)al(W.heavy + 2 * 3 * (int64_t)W.heavy_cap * (int64_t)rs, 16);
        W.params = W.tinfo + W.nstages * (int32_t)sizeof(tg::TileInfo);
        W.mbar = (int32_t)al(W.params + (int64_t)sizeof(tg::DevParams), 16);
        W.total = W.mbar + (2 * W.nstages + 2) * 8 + 32;
        s->ws_warps = s->threads_req > 0 ? s->threads_req / 32 : tg::kWsMaxConsumerWarps;
        s->ws_warps = std::max(2, std::min(tg::kWsMaxConsumerWarps, s->ws_warps)) & ~1;
        CK(tg::step_ws_prepare(s->prec, s->integrator, (size_t)W.total), "set shared memory");
        int sms = 0, dev = 0;
        CK(cudaGetDevice(&dev), "device");
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device");
        s->ctas = (int)std::min<int64_t>((int64_t)tiles_run.size(), sms);
        s->threads = (s->ws_warps + tg::kWsProducerWarps) * 32;
        s->use_ws = true;
    }
    if (s->use_pull) {
        CK(tg::step_pull_prepare(s->prec, s->integrator, (size_t)a.pull.total), "set shared memory");
        int sms = 0, dev = 0;
        CK(cudaGetDevice(&dev), "device");
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device");
        s->ctas = (int)std::min<int64_t>((int64_t)tiles_run.size(), sms);
        s->threads = (a.pull.nteams * a.pull.team_warps + 1) * 32;
    } else if (!s->use_ws) {
        if (s->smem > 227 * 1024) return s->fail(TITAN_GB300_ELIMIT, "tile does not fit in shared memory");
        s->use_async = s->kernel_req == 3;
        s->step_variant = 0;
        if (s->min_ctas_req >= 3 && s->prec != P_FP64) {
            if (s->threads > 256)
                return s->fail(TITAN_GB300_EINVAL, "3 or 4 CTAs per SM need at most 256 threads per CTA");
            s->step_variant = s->min_ctas_req == 3 ? 1 : 2;
        }
        if (s->use_async)
            CK(tg::step_async_prepare(s->prec, s->smem), "set shared memory");
        else
            CK(tg::step_prepare(s->prec, s->step_variant, s->integrator, s->smem), "set shared memory");
    }
    a.ntiles = (int32_t)tiles_run.size();
    if (P.ent_ends.size() > (size_t)INT32_MAX || P.halo.size() > (size_t)INT32_MAX)
        return s->fail(TITAN_GB300_ELIMIT, "more than 2^31 slab entries");
#define DEVCOPY(dst, vec, what)                               \
    do {                                                      \
        auto *p_ = dev_copy(s, vec, e);                       \
        if (!p_) return s->cuda_fail(e, what);                \
        dst = p_;                                             \
    } while (0)
    DEVCOPY(a.tiles, tiles_run, "upload tiles");
    if (s->use_pull) {
        DEVCOPY(a.pull_units, s->pull.units, "upload pull units");
        DEVCOPY(a.pull_ell, s->pull.ell, "upload pull columns");
    }
    if (s->use_rtiles) DEVCOPY(s->rtargs.tiles, s->rtiles, "upload resident tiles");
    if (s->use_res) {
        tg::ResPlan &R = s->rplan;
        tg::ResArgs &r = s->rargs;
        DEVCOPY(r.bin_mass_off, R.bin_mass_off, "upload bins");
        DEVCOPY(r.bin_warp_off, R.bin_warp_off, "upload bins");
        DEVCOPY(r.mass, R.mass, "upload bins");
        DEVCOPY(r.body, R.body, "upload bins");
        DEVCOPY(r.deg, R.deg, "upload bins");
        DEVCOPY(r.act_mask, R.act_mask, "upload bins");
        DEVCOPY(r.warp_rec_off, R.warp_rec_off, "upload bins");
        const size_t nrec = std::max<size_t>(1, R.words.size()) * (s->prec == P_FP64 ? 32 : 16);
        if (!(r.rec = s->mem.get(nrec, e))) return s->cuda_fail(e, "alloc resident records");
        if (!(r.act = s->mem.get(nrec, e))) return s->cuda_fail(e, "alloc resident records");
        if (!(r.next = (int *)s->mem.get(sizeof(int), e))) return s->cuda_fail(e, "alloc bin queue");
    }
    DEVCOPY(a.halo, P.halo, "upload halo");
    DEVCOPY(a.warp_inc_off, P.warp_inc_off, "upload warp offsets");
    std::vector<uint8_t> deg(np, 0);
    std::copy(P.deg.begin(), P.deg.end(), deg.begin());
    DEVCOPY(a.deg, deg, "upload degrees");
    DEVCOPY(a.inc, P.inc, "upload incidence");
    DEVCOPY(a.heavy_local, P.heavy_local, "upload heavy");
    DEVCOPY(a.heavy_inc_off, P.heavy_inc_off, "upload heavy");
    DEVCOPY(a.heavy_inc, P.heavy_inc, "upload heavy");
    DEVCOPY(s->d_old2new, P.old2new, "upload order");
    std::vector<double> bp(6 * std::max<size_t>(1, s->body_plane.size()), 0.0);
    for (size_t b = 0; b < s->body_plane.size(); b++)
        for (int c = 0; c < 6; c++) bp[6 * b + c] = s->body_plane[b][c];
    std::vector<float> bpf(bp.begin(), bp.end());
    DEVCOPY(a.body_plane, bp, "upload body planes");
    DEVCOPY(a.body_planef, bpf, "upload body planes");
#undef DEVCOPY
    const size_t E = std::max<size_t>(1, P.ent_ends.size());
    const size_t rs4 = (s->prec == P_FP64 ? 32 : 16);
    if (!(a.ent = s->mem.get(E * rs4, e))) return s->cuda_fail(e, "alloc entries");
    if (!(a.act = s->mem.get(E * rs4, e))) return s->cuda_fail(e, "alloc actuation");
    if (!(a.mass = s->mem.get(np * rs, e))) return s->cuda_fail(e, "alloc mass");
    if (!(a.flags = (const uint8_t *)s->mem.get(np, e))) return s->cuda_fail(e, "alloc flags");
    if (!(a.ext = s->mem.get(3 * np * rs, e))) return s->cuda_fail(e, "alloc ext");
    if (!(a.drag = (const int32_t *)s->mem.get(np * 4, e))) return s->cuda_fail(e, "alloc drag");
    if (!(a.lc_ptr = (const int32_t *)s->mem.get((np + 1) * 4, e))) return s->cuda_fail(e, "alloc lc");
    if (!(a.state0 = s->mem.get(s->comps() * np * rs, e))) return s->cuda_fail(e, "alloc state");
    if (!(a.state1 = s->mem.get(s->comps() * np * rs, e))) return s->cuda_fail(e, "alloc state");
    if (!(a.acc = s->mem.get(3 * np * rs, e))) return s->cuda_fail(e, "alloc acc");
    if (!(a.tbuf = (double *)s->mem.get(2 * sizeof(double), e))) return s->cuda_fail(e, "alloc time");
    if (s->use_rtiles) {
        if (!(s->rtargs.t0 = (const double *)s->mem.get(sizeof(double), e))) return s->cuda_fail(e, "alloc time");
        if (!s->side_stream) CK(cudaStreamCreateWithFlags(&s->side_stream, cudaStreamNonBlocking), "create stream");
        if (!s->ev_fork) CK(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming), "create event");
        if (!s->ev_join) CK(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming), "create event");
    }
    if (!(s->dprm = (tg::DevParams *)s->mem.get(sizeof(tg::DevParams), e))) return s->cuda_fail(e, "alloc params");
    a.prm = s->dprm;
    if (!(s->d_err = (int *)s->mem.get(sizeof(int), e))) return s->cuda_fail(e, "alloc error flag");
    CK(cudaMemset(s->d_err, 0, sizeof(int)), "clear error flag");
    a.err = s->d_err;
    if (!(s->d_xfer = (double *)s->mem.get(9 * (size_t)s->n * 8, e))) return s->cuda_fail(e, "alloc staging");
    if (!(s->d_idx = (int64_t *)s->mem.get((size_t)s->n * 8, e))) return s->cuda_fail(e, "alloc staging");
    CK(cudaMallocHost(&s->h_xfer, 9 * (size_t)s->n * 8), "alloc pinned staging");
    CK(cudaMemset(a.state0, 0, s->comps() * np * rs), "clear state");
    CK(cudaMemset(a.state1, 0, s->comps() * np * rs), "clear state");
    CK(cudaMemset(a.acc, 0, 3 * np * rs), "clear acc");

    int rc = upload_entries(s);
    if (rc) return rc;
    rc = upload_mass_attrs(s);
    if (rc) return rc;
    // positions / velocities into both ping-pong buffers
    std::memcpy(s->h_xfer, s->pos.data(), 3 * s->n * 8);
    std::memcpy(s->h_xfer + 3 * s->n, s->vel.data(), 3 * s->n * 8);
    CK(cudaMemcpy(s->d_xfer, s->h_xfer, 6 * s->n * 8, cudaMemcpyHostToDevice), "upload state");
    tg::XferArgs x{};
    x.old2new = s->d_old2new;
    x.count = s->n;
    x.npad = np;
    x.state0 = a.state0;
    x.state1 = a.state1;
    x.acc = a.acc;
    x.ipos = s->d_xfer;
    x.ivel = s->d_xfer + 3 * s->n;
    CK(tg::launch_scatter(s->prec, x, s->stream), "scatter state");
    s->parity = 0;
    rc = upload_params(s);
    if (rc) return rc;
    CK(cudaStreamSynchronize(s->stream), "start");
    return TITAN_GB300_OK;
}

// Downloads positions/velocities into the host mirror (creation order).
int pull_state(titan_gb300_sim *s) {
    tg::XferArgs x{};
    x.old2new = s->d_old2new;
    x.count = s->n;
    x.npad = s->npad;
    x.state0 = s->args.state0;
    x.state1 = s->args.state1;
    x.acc = s->args.acc;
    x.parity = s->parity;
    x.pos = s->d_xfer;
    x.vel = s->d_xfer + 3 * s->n;
    CK(tg::launch_gather(s->prec, x, s->stream), "gather state");
    CK(cudaMemcpyAsync(s->h_xfer, s->d_xfer, 6 * s->n * 8, cudaMemcpyDeviceToHost, s->stream), "download");
    CK(cudaStreamSynchronize(s->stream), "download");
    std::memcpy(s->pos.data(), s->h_xfer, 3 * s->n * 8);
    std::memcpy(s->vel.data(), s->h_xfer + 3 * s->n, 3 * s->n * 8);
    return TITAN_GB300_OK;
}

// Per-mass local time: the reference adds dt to each free mass every step
// (src/sim.cu:1165); replay those additions from the mass's last upload.
void mass_times(titan_gb300_sim *s, const int64_t *idx, int64_t count, double *T) {
    std::map<std::pair<uint64_t, int64_t>, double> memo;
    for (int64_t q = 0; q < count; q++) {
        int64_t i = idx ? idx[q] : q;
        if (!s->fixed.empty() && s->fixed[i]) {
            T[q] = s->mT0[i];
            continue;
        }
        uint64_t bits;
        std::memcpy(&bits, &s->mT0[i], 8);
        auto key = std::make_pair(bits, s->mTstep[i]);
        auto it = memo.find(key);
        if (it != memo.end()) {
            T[q] = it->second;
            continue;
        }
        double t = s->mT0[i];
        int64_t st = s->mTstep[i];
        for (size_t r = 0; r < s->dt_log.size(); r++) {
            int64_t b = s->dt_log[r].first;
            int64_t e = r + 1 < s->dt_log.size() ? s->dt_log[r + 1].first : s->steps;
            double d = s->dt_log[r].dt;
            if (s->dt_log[r].halves == 2) {  // RK2: mass.T += 0.5 * dt twice per step
                const double h = 0.5 * d;
                for (int64_t z = std::max(b, st); z < e; z++) {
                    t = t + h;
                    t = t + h;
                }
                continue;
            }
            for (int64_t z = std::max(b, st); z < e; z++) t = t + d;
        }
        memo[key] = t;
        T[q] = t;
    }
}

cudaGraphExec_t get_graph(titan_gb300_sim *s, int len, int parity, cudaError_t &e) {
    auto key = std::make_pair(len, parity);
    auto it = s->graphs.find(key);
    if (it != s->graphs.end()) return it->second;
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return nullptr;
    int p = parity;
    cudaError_t el = cudaSuccess;  // the first launch refused while capturing
    for (int i = 0; i < len; i++)
        for (int q = 0; q < s->passes(); q++) {
            const cudaError_t r = s->launch(p, 0, q);
            if (el == cudaSuccess) el = r;
            p ^= 1;
        }
    e = cudaStreamEndCapture(s->stream, &g);
    if (e == cudaSuccess && el != cudaSuccess) {
        cudaGraphDestroy(g);
        e = el;
    }
    if (e != cudaSuccess) return nullptr;
    cudaGraphExec_t ex = nullptr;
    e = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return nullptr;
    s->graphs[key] = ex;
    return ex;
}

bool ensure_device(titan_gb300_sim *s) { return cudaSetDevice(s->device) == cudaSuccess; }

// After a synchronisation: did a step kernel give up a bounded wait?
int check_kernel_error(titan_gb300_sim *s) {
    if (!s->d_err) return TITAN_GB300_OK;
    int flag = 0;
    CK(cudaMemcpy(&flag, s->d_err, sizeof(int), cudaMemcpyDeviceToHost), "read error flag");
    if (flag) {
        cudaMemset(s->d_err, 0, sizeof(int));
        return s->fail(TITAN_GB300_ETIMEOUT, "a step kernel's bounded wait for its shared-memory copies timed out");
    }
    return TITAN_GB300_OK;
}

}  // namespace

namespace tg {

int serve_begin(titan_gb300_sim *s, int device, int precision, size_t tile_smem, ServeScene &v, std::string &why) {
    if (!s->started) return why = "the scene has not started", TITAN_GB300_ESTATE;
    if (s->serving) return why = "the scene is already with a server", TITAN_GB300_ESTATE;
    if (s->device != device || s->prec != precision)
        return why = "the scene's device or precision differs from the server's", TITAN_GB300_EINVAL;
    if (s->integrator != INTEG_EULER) return why = "the server steps symplectic Euler only", TITAN_GB300_EINVAL;
    if (s->use_res || s->use_rtiles || s->args.ntiles <= 0)
        return why = "start the scene with resident tiles and bins off (set_resident 0)", TITAN_GB300_EINVAL;
    size_t need = 0;
    for (const TileInfo &ti : tile_infos(s->plan))
        need = std::max(need, tile_smem_bytes(s->prec, ti.nm + ti.nh, ti.ne + 1, ti.nheavy));
    if (need > tile_smem)
        return why = "a tile needs more shared memory than the server has (plan smaller tiles)", TITAN_GB300_ELIMIT;
    if (!ensure_device(s)) return why = "cudaSetDevice failed", TITAN_GB300_ECUDA;
    const cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return why = std::string("scene stream: ") + cudaGetErrorString(e), TITAN_GB300_ECUDA;
    s->serving = true;
    v.args = &s->args;
    v.parity = s->parity;
    return TITAN_GB300_OK;
}

void serve_end(titan_gb300_sim *s, int64_t nsteps) {
    s->serving = false;
    if (nsteps <= 0) return;
    s->parity ^= (int)(nsteps & 1);
    for (int64_t i = 0; i < nsteps; i++) s->T = s->T + s->dt;  // src/sim.cu:1590
    s->steps += nsteps;
}

}  // namespace tg

// Status of a C++ exception that reached an entry point (a host allocation
// that failed, or a library error): the C ABI throws nothing, and the
// message goes to the handle when there is one.
static int host_exception(titan_gb300_sim *s) noexcept {
    int code = TITAN_GB300_EINVAL;
    std::string msg = "host error";
    try {
        throw;
    } catch (const std::bad_alloc &) {
        code = TITAN_GB300_ENOMEM;
        msg = "host memory exhausted";
    } catch (const std::exception &e) {
        try {
            msg = std::string("host error: ") + e.what();
        } catch (...) {
        }
    } catch (...) {
    }
    if (s) {
        try {
            s->err = msg;
        } catch (...) {
        }
    }
    return code;
}

extern "C" {

const char *titan_gb300_version(void) { return "titan_gb300 0.1 (sm_103a)"; }

int titan_gb300_create(titan_gb300_sim **out, int device, int precision) try {
    if (!out) return TITAN_GB300_EINVAL;
    *out = nullptr;
    if (precision < 0 || precision > 2 || device < 0) return TITAN_GB300_EINVAL;
    // No CUDA call here: the device and stream are taken at start(), so a
    // scene can be built and planned on a host without a GPU.
    auto *s = new (std::nothrow) titan_gb300_sim();
    if (!s) return TITAN_GB300_ENOMEM;
    s->device = device;
    s->prec = precision;
    *out = s;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(nullptr);
}

void titan_gb300_destroy(titan_gb300_sim *s) {
    if (!s) return;
    if (s->stream) ensure_device(s);
    delete s;
}

int titan_gb300_set_launch(titan_gb300_sim *s, int threads_per_cta) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (threads_per_cta != 0 && (threads_per_cta < 64 || threads_per_cta > 512 || threads_per_cta % 32))
        return s->fail(TITAN_GB300_EINVAL, "threads per CTA must be 0 or a multiple of 32 in [64, 512]");
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "set the launch shape before start");
    s->threads_req = threads_per_cta;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_occupancy(titan_gb300_sim *s, int min_ctas_per_sm) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (min_ctas_per_sm < 0 || min_ctas_per_sm > 4 || min_ctas_per_sm == 2)
        return s->fail(TITAN_GB300_EINVAL, "minimum CTAs per SM must be 0, 1, 3 or 4");
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "set the occupancy before start");
    s->min_ctas_req = min_ctas_per_sm;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_kernel(titan_gb300_sim *s, int variant) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (variant < 0 || variant > 6 || variant == 2 || variant == 5)
        return s->fail(TITAN_GB300_EINVAL, "kernel variant must be 0, 1, 3, 4 or 6");
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "choose the kernel before start");
    s->kernel_req = variant;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_kernel_info(const titan_gb300_sim *s, int64_t out[4]) {
    if (!s || !out) return TITAN_GB300_EINVAL;
    if (s->use_rtiles && s->args.ntiles == 0) {
        out[0] = 5;
        out[1] = s->rtargs.ntiles;
        out[2] = s->rt_threads;
        out[3] = (int64_t)s->rt_smem;
        return TITAN_GB300_OK;
    }
    out[0] = s->use_pull ? 6 : (s->use_async ? 3 : (s->use_ws ? 4 : 1));
    out[1] = (s->use_ws || s->use_pull) ? s->ctas : s->args.ntiles;
    out[2] = s->threads;
    out[3] = s->use_pull ? s->args.pull.total : (s->use_ws ? s->args.ws.total : (int64_t)s->smem);
    return TITAN_GB300_OK;
}

int titan_gb300_set_resident(titan_gb300_sim *s, int mode, int bin_masses, int threads_per_cta) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (mode < -1 || mode > 2) return s->fail(TITAN_GB300_EINVAL, "resident mode must be -1, 0, 1 or 2");
    if (bin_masses < 0 || bin_masses > 32767) return s->fail(TITAN_GB300_EINVAL, "bin size must be in [0, 32767]");
    if (threads_per_cta != 0 && (threads_per_cta < 64 || threads_per_cta > 512 || threads_per_cta % 32))
        return s->fail(TITAN_GB300_EINVAL, "threads per CTA must be 0 or a multiple of 32 in [64, 512]");
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "configure resident bins before start");
    s->res_mode = mode;
    s->res_bin_req = bin_masses;
    s->res_threads_req = threads_per_cta;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_resident_info(const titan_gb300_sim *s, int64_t out[8]) {
    if (!s || !out) return TITAN_GB300_EINVAL;
    std::memset(out, 0, 8 * sizeof(int64_t));
    if (s->use_rtiles) {
        out[0] = 2;
        out[1] = (int64_t)s->rtiles.size();
        std::vector<int32_t> bodies;
        int64_t nm = 0, cap = 0;
        for (const tg::TileInfo &ti : s->rtiles) {
            bodies.push_back(ti.body);
            nm += ti.nm;
            cap = std::max<int64_t>(cap, ti.nm);
        }
        std::sort(bodies.begin(), bodies.end());
        out[2] = (int64_t)(std::unique(bodies.begin(), bodies.end()) - bodies.begin());
        out[3] = nm;
        out[4] = cap;
        out[5] = s->rt_threads;
        out[6] = (int64_t)s->rtiles.size();
        out[7] = (int64_t)s->rt_smem;
        return TITAN_GB300_OK;
    }
    if (!s->use_res) return TITAN_GB300_OK;
    out[0] = 1;
    out[1] = s->rplan.nbins;
    out[2] = s->rplan.nbodies;
    out[3] = s->rplan.nmasses;
    out[4] = s->rargs.cap;
    out[5] = s->res_threads;
    out[6] = s->res_ctas;
    out[7] = (int64_t)tg::resident_smem_bytes(s->prec, s->rargs.cap);
    return TITAN_GB300_OK;
}

int titan_gb300_adopt_plan(titan_gb300_sim *s, const titan_gb300_sim *src) try {
    if (!s || !src) return TITAN_GB300_EINVAL;
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "adopt a plan before start");
    if (src->plan.ntiles <= 0) return s->fail(TITAN_GB300_EINVAL, "the source handle has no plan");
    auto flags = [](const titan_gb300_sim *h, int64_t i) { return !h->fixed.empty() && h->fixed[i] != 0; };
    auto act = [](const titan_gb300_sim *h, int64_t j) { return !h->type.empty() && h->type[j] >= 2; };
    bool same = s->prec == src->prec && s->n == src->n && s->ns == src->ns && s->left == src->left &&
                s->right == src->right && s->body_ptr == src->body_ptr && s->kernel_req == src->kernel_req;
    for (int64_t i = 0; same && i < s->n; i++) same = flags(s, i) == flags(src, i);
    for (int64_t j = 0; same && j < s->ns; j++) same = act(s, j) == act(src, j);
    if (!same)
        return s->fail(TITAN_GB300_EINVAL,
                       "adopt_plan needs the same precision, kernel form, masses, springs, fixed masses, "
                       "actuated springs and bodies");
    s->plan = src->plan;
    s->plan_tile = src->plan_tile;
    s->plan_req = src->plan_req;
    s->plan_adopted = true;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_plan_host(titan_gb300_sim *s, int tile_masses) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "plan_host is for scenes that have not started");
    if (s->n <= 0) return s->fail(TITAN_GB300_EINVAL, "no masses");
    tg::PlanInput in;
    std::string why = plan_scene(s, tile_masses, in);
    if (!why.empty()) return s->fail(TITAN_GB300_ELIMIT, why);
    s->plan_tile = in.tile_cap;
    s->plan_adopted = false;
    s->rplan = tg::ResPlan();
    const int cap = resident_cap(s);
    if (cap > 0) tg::build_resident(in, s->plan, cap, cap, s->rplan);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int64_t titan_gb300_plan_table(const titan_gb300_sim *s, int table, void *out) {
    if (!s) return -1;
    const tg::Plan &P = s->plan;
    auto put = [&](const auto &v) -> int64_t {
        if (out && !v.empty()) std::memcpy(out, v.data(), v.size() * sizeof(v[0]));
        return (int64_t)v.size();
    };
    switch (table) {
        case TITAN_GB300_T_NEW2OLD: return put(P.new2old);
        case TITAN_GB300_T_TILE_MASS_OFF: return put(P.tile_mass_off);
        case TITAN_GB300_T_TILE_HALO_OFF: return put(P.tile_halo_off);
        case TITAN_GB300_T_HALO: return put(P.halo);
        case TITAN_GB300_T_TILE_ENT_OFF: return put(P.tile_ent_off);
        case TITAN_GB300_T_TILE_NACT: return put(P.tile_nact);
        case TITAN_GB300_T_ENT_ENDS: return put(P.ent_ends);
        case TITAN_GB300_T_ENT_SPRING: return put(P.ent_spring);
        case TITAN_GB300_T_TILE_WARP_OFF: return put(P.tile_warp_off);
        case TITAN_GB300_T_WARP_INC_OFF: return put(P.warp_inc_off);
        case TITAN_GB300_T_DEG: return put(P.deg);
        case TITAN_GB300_T_INC: return put(P.inc);
        case TITAN_GB300_T_TILE_HEAVY_OFF: return put(P.tile_heavy_off);
        case TITAN_GB300_T_HEAVY_LOCAL: return put(P.heavy_local);
        case TITAN_GB300_T_HEAVY_INC_OFF: return put(P.heavy_inc_off);
        case TITAN_GB300_T_HEAVY_INC: return put(P.heavy_inc);
        case TITAN_GB300_T_BODY_OF_TILE: return put(P.body_of_tile);
        case TITAN_GB300_T_TILE_NH: return put(P.tile_nh);
        case TITAN_GB300_T_RES_BIN_MASS_OFF: return put(s->rplan.bin_mass_off);
        case TITAN_GB300_T_RES_BIN_WARP_OFF: return put(s->rplan.bin_warp_off);
        case TITAN_GB300_T_RES_MASS: return put(s->rplan.mass);
        case TITAN_GB300_T_RES_BODY: return put(s->rplan.body);
        case TITAN_GB300_T_RES_DEG: return put(s->rplan.deg);
        case TITAN_GB300_T_RES_ACT_MASK: return put(s->rplan.act_mask);
        case TITAN_GB300_T_RES_WARP_REC_OFF: return put(s->rplan.warp_rec_off);
        case TITAN_GB300_T_RES_WORDS: return put(s->rplan.words);
        case TITAN_GB300_T_RES_REC_SPRING: return put(s->rplan.rec_spring);
        case TITAN_GB300_T_RES_RESIDENT: return put(s->rplan.resident);
        default: return -1;
    }
}

const char *titan_gb300_last_error(const titan_gb300_sim *s) {
    return s ? s->err.c_str() : "null handle";
}

int titan_gb300_set_masses(titan_gb300_sim *s, int64_t n, const double *pos, const double *vel,
                           const double *m, const double *ext, const uint8_t *fixed, const double *drag) try {
    if (!s) return TITAN_GB300_EINVAL;
    s->plan_adopted = false;  // the topology may change
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "masses can only be replaced before start");
    if (n <= 0 || !pos || !m) return s->fail(TITAN_GB300_EINVAL, "need n > 0, pos and m");
    s->n = n;
    s->pos.assign(pos, pos + 3 * n);
    s->vel.assign(3 * n, 0.0);
    if (vel) s->vel.assign(vel, vel + 3 * n);
    s->m.assign(m, m + n);
    s->ext.clear();
    if (ext) s->ext.assign(ext, ext + 3 * n);
    s->fixed.clear();
    if (fixed) s->fixed.assign(fixed, fixed + n);
    s->drag.clear();
    if (drag) {
        s->drag.resize(n);
        for (int64_t i = 0; i < n; i++) s->drag[i] = (int32_t)drag[i];  // object.h:213 truncation
    }
    s->lc_ptr.clear();
    s->lc_type.clear();
    s->lc_rec.clear();
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_springs(titan_gb300_sim *s, int64_t n, const int32_t *left, const int32_t *right,
                            const double *k, const double *rest, const double *damping,
                            const int32_t *type, const double *omega, const double *amp,
                            const double *phase) try {
    if (!s) return TITAN_GB300_EINVAL;
    s->plan_adopted = false;  // the topology may change
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "springs can only be replaced before start");
    if (n < 0 || (n > 0 && (!left || !right || !k || !rest))) return s->fail(TITAN_GB300_EINVAL, "bad springs");
    s->ns = n;
    s->left.assign(left, left + n);
    s->right.assign(right, right + n);
    s->k.assign(k, k + n);
    s->rest.assign(rest, rest + n);
    s->damping.assign(n, 0.0);
    if (damping) s->damping.assign(damping, damping + n);
    s->type.clear();
    if (type) {
        s->type.assign(type, type + n);
        for (int32_t t : s->type)
            if (t < 0 || t > 3) return s->fail(TITAN_GB300_EINVAL, "spring type must be 0..3");
    }
    s->omega.clear();
    if (omega) s->omega.assign(omega, omega + n);
    s->amp.clear();
    if (amp) s->amp.assign(amp, amp + n);
    s->phase.clear();
    if (phase) s->phase.assign(phase, phase + n);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_local_constraints(titan_gb300_sim *s, const int64_t *mass_ptr, const int32_t *type,
                                      const double *vec, const double *num) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "set local constraints before start");
    if (s->n <= 0 || !mass_ptr) return s->fail(TITAN_GB300_EINVAL, "set masses first");
    int64_t nr = mass_ptr[s->n];
    if (mass_ptr[0] != 0 || nr < 0) return s->fail(TITAN_GB300_EINVAL, "bad record offsets");
    static const int order[4] = {1, 2, 0, 3};  // contact, ball, constraint plane, direction
    s->lc_ptr.assign(s->n + 1, 0);
    s->lc_type.clear();
    s->lc_rec.clear();
    for (int64_t i = 0; i < s->n; i++) {
        if (mass_ptr[i + 1] < mass_ptr[i]) return s->fail(TITAN_GB300_EINVAL, "bad record offsets");
        for (int o = 0; o < 4; o++)
            for (int64_t r = mass_ptr[i]; r < mass_ptr[i + 1]; r++) {
                if (type[r] != order[o]) continue;
                double v[3] = {vec[3 * r], vec[3 * r + 1], vec[3 * r + 2]};
                if (type[r] != TITAN_GB300_BALL) {  // constructors normalise (object.cu:60,109,127)
                    double nn = norm3(v);
                    if (nn == 0.0) return s->fail(TITAN_GB300_EINVAL, "zero constraint vector");
                    for (double &c : v) c = c / nn;
                }
                s->lc_type.push_back(type[r]);
                s->lc_rec.insert(s->lc_rec.end(), {v[0], v[1], v[2], num[r]});
            }
        s->lc_ptr[i + 1] = (int64_t)s->lc_type.size();
    }
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_add_plane(titan_gb300_sim *s, const double normal[3], double offset, double fk, double fs) try {
    if (!s || !normal) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if ((int)s->planes.size() >= tg::kMaxPlanes) return s->fail(TITAN_GB300_ELIMIT, "at most 16 global planes");
    double nn = norm3(normal);
    if (!(nn > 0)) return s->fail(TITAN_GB300_EINVAL, "zero plane normal");
    s->planes.push_back({normal[0] / nn, normal[1] / nn, normal[2] / nn, offset, fk, fs});
    if (s->started) return upload_params(s);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_add_ball(titan_gb300_sim *s, const double center[3], double radius) try {
    if (!s || !center) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if ((int)s->balls.size() >= tg::kMaxBalls) return s->fail(TITAN_GB300_ELIMIT, "at most 16 global balls");
    s->balls.push_back({center[0], center[1], center[2], radius});
    if (s->started) return upload_params(s);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_clear_constraints(titan_gb300_sim *s) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    s->planes.clear();
    s->balls.clear();
    if (s->started) return upload_params(s);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_integrator(titan_gb300_sim *s, int kind) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (kind < tg::INTEG_EULER || kind > tg::INTEG_RK2)
        return s->fail(TITAN_GB300_EINVAL, "integrator must be 0 (Euler), 1 (Verlet) or 2 (RK2)");
    if (kind == s->integrator) return TITAN_GB300_OK;
    if (!s->started) {
        s->integrator = kind;
        return TITAN_GB300_OK;
    }
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    CK(cudaStreamSynchronize(s->stream), "set integrator");
    const bool was_res = s->use_res || s->use_rtiles;
    s->integrator = kind;
    s->dt_log.push_back({s->steps, s->dt, s->passes()});
    s->drop_graphs();
    if (was_res) {  // resident bins and tiles run Euler only: rebuild without them
        int rc = pull_state(s);
        if (rc) return rc;
        return build_device(s);
    }
    // the kernels of the new integrator need their shared-memory limit
    if (s->use_pull)
        CK(tg::step_pull_prepare(s->prec, kind, (size_t)s->args.pull.total), "set shared memory");
    else if (s->use_ws)
        CK(tg::step_ws_prepare(s->prec, kind, (size_t)s->args.ws.total), "set shared memory");
    else if (!s->use_async)
        CK(tg::step_prepare(s->prec, s->step_variant, kind, s->smem), "set shared memory");
    return upload_params(s);
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_time_step(titan_gb300_sim *s, double dt) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!(dt > 0)) return s->fail(TITAN_GB300_EINVAL, "Cannot set time step to negative or zero value.");
    s->dt = dt;
    if (s->started) {
        s->dt_log.push_back({s->steps, dt, s->passes()});
        return upload_params(s);
    }
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

double titan_gb300_get_time_step(const titan_gb300_sim *s) { return s ? s->dt : 0.0; }

int titan_gb300_set_global_acc(titan_gb300_sim *s, const double g[3]) try {
    if (!s || !g) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    for (int c = 0; c < 3; c++) s->g[c] = g[c];
    if (s->started) return upload_params(s);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_bodies(titan_gb300_sim *s, int64_t nbodies, const int64_t *mass_ptr) try {
    if (!s) return TITAN_GB300_EINVAL;
    s->plan_adopted = false;  // the topology may change
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "set bodies before start");
    if (nbodies <= 0 || !mass_ptr || mass_ptr[0] != 0 || mass_ptr[nbodies] != s->n)
        return s->fail(TITAN_GB300_EINVAL, "body ranges must cover all masses");
    for (int64_t b = 0; b < nbodies; b++)
        if (mass_ptr[b + 1] <= mass_ptr[b]) return s->fail(TITAN_GB300_EINVAL, "empty body");
    s->body_ptr.assign(mass_ptr, mass_ptr + nbodies + 1);
    s->body_plane.assign(nbodies, {0, 0, 1, 0, 0, 0});
    s->body_has_plane.assign(nbodies, 0);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_body_plane(titan_gb300_sim *s, int64_t body, const double normal[3], double offset,
                               double fk, double fs) try {
    if (!s || !normal) return TITAN_GB300_EINVAL;
    if (s->started) return s->fail(TITAN_GB300_ESTATE, "set body planes before start");
    if (body < 0 || body >= (int64_t)s->body_plane.size()) return s->fail(TITAN_GB300_EINVAL, "no such body");
    double nn = norm3(normal);
    if (!(nn > 0)) return s->fail(TITAN_GB300_EINVAL, "zero plane normal");
    s->body_plane[body] = {normal[0] / nn, normal[1] / nn, normal[2] / nn, offset, fk, fs};
    s->body_has_plane[body] = 1;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_start(titan_gb300_sim *s, int tile_masses) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->n <= 0)
        return s->fail(TITAN_GB300_EINVAL, "No masses have been added. Please add masses before starting the simulation.");
    if (!(s->dt > 0)) return s->fail(TITAN_GB300_EINVAL, "invalid time step");
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    if (!s->stream) CK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "create stream");
    s->tile_masses = tile_masses;
    s->T = 0.0;
    s->steps = 0;
    s->dt_log.assign(1, {0, s->dt, s->passes()});
    s->mT0.assign(s->n, 0.0);
    s->mTstep.assign(s->n, 0);
    int rc = build_device(s);
    if (rc) return rc;
    s->started = true;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_step(titan_gb300_sim *s, int64_t nsteps) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (nsteps < 0) return s->fail(TITAN_GB300_EINVAL, "negative step count");
    if (nsteps == 0) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    cudaError_t e = cudaSuccess;
    if (s->use_res)
        CK(tg::launch_resident(s->prec, s->args, s->rargs, s->res_ctas, s->res_threads, s->parity, nsteps, 1,
                               s->args.ntiles == 0, s->stream),
           "launch resident bins");
    bool joined = true;
    if (s->use_rtiles) {
        // the first step's time, copied before per-step kernels advance the record
        CK(cudaMemcpyAsync(const_cast<double *>(s->rtargs.t0), s->args.tbuf + s->parity, sizeof(double),
                           cudaMemcpyDeviceToDevice, s->stream),
           "launch resident tiles");
        if (s->args.ntiles == 0) {
            CK(tg::launch_tile_resident(s->prec, s->args, s->rtargs, s->rt_mpt, s->rt_threads, s->rt_smem,
                                        s->parity, nsteps, 1, s->stream),
               "launch resident tiles");
            CK(tg::launch_advance_time(s->args, s->parity, nsteps, s->stream), "advance time");
        } else {  // beside the per-step kernels: disjoint masses
            CK(cudaEventRecord(s->ev_fork, s->stream), "launch resident tiles");
            CK(cudaStreamWaitEvent(s->side_stream, s->ev_fork, 0), "launch resident tiles");
            CK(tg::launch_tile_resident(s->prec, s->args, s->rtargs, s->rt_mpt, s->rt_threads, s->rt_smem,
                                        s->parity, nsteps, 1, s->side_stream),
               "launch resident tiles");
            CK(cudaEventRecord(s->ev_join, s->side_stream), "launch resident tiles");
            joined = false;
        }
    }
    if (s->args.ntiles == 0) {
        s->parity ^= (int)(nsteps & 1);
        for (int64_t i = 0; i < nsteps; i++) s->T = s->T + s->dt;  // src/sim.cu:1590
        s->steps += nsteps;
        return TITAN_GB300_OK;
    }
    const int P = s->passes();
    const int rc = [&]() -> int {
        int64_t rem = nsteps - 1;
        while (rem > 0) {
            int len = (int)std::min<int64_t>(rem, kChunk);
            cudaGraphExec_t g = get_graph(s, len, s->parity, e);
            if (!g) return s->cuda_fail(e, "build step graph");
            CK(cudaGraphLaunch(g, s->stream), "launch step graph");
            s->parity ^= ((len * P) & 1);
            rem -= len;
        }
        for (int q = 0; q < P; q++) {  // the last step also writes the accelerations
            CK(s->launch(s->parity, q == P - 1, q), "launch step");
            s->parity ^= 1;
        }
        return TITAN_GB300_OK;
    }();
    // later work on the handle's stream sees the resident tiles' results
    if (!joined) CK(cudaStreamWaitEvent(s->stream, s->ev_join, 0), "join resident tiles");
    if (rc) return rc;
    if (P == 2) {
        const double h = 0.5 * s->dt;
        for (int64_t i = 0; i < nsteps; i++) {  // src/sim.cu:1574-1583
            s->T = s->T + h;
            s->T = s->T + h;
        }
    } else {
        for (int64_t i = 0; i < nsteps; i++) s->T = s->T + s->dt;  // src/sim.cu:1590
    }
    s->steps += nsteps;
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_prepare_steps(titan_gb300_sim *s, int64_t nsteps) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (nsteps < 0) return s->fail(TITAN_GB300_EINVAL, "negative step count");
    if (s->args.ntiles == 0 || nsteps <= 1) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    // the same chunk sequence step(nsteps) replays, from the current parity
    cudaError_t e = cudaSuccess;
    const int P = s->passes();
    int parity = s->parity;
    for (int64_t rem = nsteps - 1; rem > 0;) {
        const int len = (int)std::min<int64_t>(rem, kChunk);
        if (!get_graph(s, len, parity, e)) return s->cuda_fail(e, "build step graph");
        parity ^= ((len * P) & 1);
        rem -= len;
    }
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_synchronize(titan_gb300_sim *s) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (!s->stream) return TITAN_GB300_OK;
    CK(cudaStreamSynchronize(s->stream), "synchronize");
    return check_kernel_error(s);
} catch (...) {
    return host_exception(s);
}

int titan_gb300_poll(titan_gb300_sim *s) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (!s->stream) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    const cudaError_t e = cudaStreamQuery(s->stream);
    if (e == cudaErrorNotReady) return TITAN_GB300_EBUSY;
    if (e != cudaSuccess) return s->cuda_fail(e, "poll");
    return check_kernel_error(s);
} catch (...) {
    return host_exception(s);
}

int titan_gb300_wait(titan_gb300_sim *s, double timeout_ms) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (!(timeout_ms >= 0)) return s->fail(TITAN_GB300_EINVAL, "timeout must be >= 0");
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const int rc = titan_gb300_poll(s);
        if (rc != TITAN_GB300_EBUSY) return rc;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (ms >= timeout_ms) return s->fail(TITAN_GB300_ETIMEOUT, "queued steps still running at the time limit");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
} catch (...) {
    return host_exception(s);
}

int titan_gb300_export_vertices(titan_gb300_sim *s, float *out, int out_on_device) try {
    if (!s || !out) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    tg::XferArgs x{};
    x.old2new = s->d_old2new;
    x.count = s->n;
    x.npad = s->npad;
    x.state0 = s->args.state0;
    x.state1 = s->args.state1;
    x.acc = s->args.acc;
    x.parity = s->parity;
    if (out_on_device) {
        CK(tg::launch_export_f32(s->prec, x, out, s->stream), "export vertices");
        return TITAN_GB300_OK;
    }
    // host buffer: through the staging area (9n doubles >= 3n floats)
    float *d = reinterpret_cast<float *>(s->d_xfer);
    CK(tg::launch_export_f32(s->prec, x, d, s->stream), "export vertices");
    CK(cudaMemcpyAsync(out, d, 3 * (size_t)s->n * sizeof(float), cudaMemcpyDeviceToHost, s->stream),
       "export vertices");
    CK(cudaStreamSynchronize(s->stream), "export vertices");
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_export_indices(titan_gb300_sim *s, uint32_t *out, int out_on_device) try {
    if (!s || !out) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    std::vector<uint32_t> idx(2 * (size_t)s->ns, 0);
    for (int64_t j = 0; j < s->ns; j++) {
        const int32_t l = s->left[j], r = s->right[j];
        if (l < 0 || r < 0 || l >= s->n || r >= s->n) continue;  // detached: (0, 0)
        idx[2 * j] = (uint32_t)l;
        idx[2 * j + 1] = (uint32_t)r;
    }
    if (!out_on_device) {
        if (!idx.empty()) std::memcpy(out, idx.data(), idx.size() * sizeof(uint32_t));
        return TITAN_GB300_OK;
    }
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    if (!idx.empty())
        CK(cudaMemcpy(out, idx.data(), idx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "export indices");
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

double titan_gb300_time(const titan_gb300_sim *s) { return s ? s->T : 0.0; }

int64_t titan_gb300_device_bytes(const titan_gb300_sim *s) { return s ? (int64_t)s->mem.total : 0; }

void *titan_gb300_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (bytes == 0 || cudaMallocHost(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void titan_gb300_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

int titan_gb300_set_time(titan_gb300_sim *s, double T) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    s->T = T;
    if (!s->started) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    return upload_params(s);
} catch (...) {
    return host_exception(s);
}
int64_t titan_gb300_steps(const titan_gb300_sim *s) { return s ? s->steps : 0; }

int titan_gb300_get_masses(titan_gb300_sim *s, int64_t count, const int64_t *idx, double *pos, double *vel,
                           double *acc, double *T) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (count < 0 || count > s->n) return s->fail(TITAN_GB300_EINVAL, "bad count");
    if (idx)
        for (int64_t q = 0; q < count; q++)
            if (idx[q] < 0 || idx[q] >= s->n) return s->fail(TITAN_GB300_EINVAL, "mass index out of range");
    if (count == 0) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    tg::XferArgs x{};
    x.old2new = s->d_old2new;
    x.count = count;
    x.npad = s->npad;
    x.state0 = s->args.state0;
    x.state1 = s->args.state1;
    x.acc = s->args.acc;
    x.parity = s->parity;
    if (idx) {
        CK(cudaMemcpyAsync(s->d_idx, idx, count * 8, cudaMemcpyHostToDevice, s->stream), "upload index");
        x.idx = s->d_idx;
    }
    x.pos = pos ? s->d_xfer : nullptr;
    x.vel = vel ? s->d_xfer + 3 * count : nullptr;
    x.accout = acc ? s->d_xfer + 6 * count : nullptr;
    // only the requested arrays come back: into a pinned caller buffer by
    // DMA directly, else through the handle's pinned staging buffer
    double *outs[3] = {pos, vel, acc};
    bool direct[3] = {false, false, false};
    if (pos || vel || acc) {
        CK(tg::launch_gather(s->prec, x, s->stream), "gather");
        for (int q = 0; q < 3; q++) {
            if (!outs[q]) continue;
            direct[q] = host_pinned(outs[q]);
            double *dst = direct[q] ? outs[q] : s->h_xfer + 3 * q * count;
            CK(cudaMemcpyAsync(dst, s->d_xfer + 3 * q * count, 3 * count * 8, cudaMemcpyDeviceToHost, s->stream),
               "download");
        }
    }
    CK(cudaStreamSynchronize(s->stream), "download");
    if (int rc = check_kernel_error(s)) return rc;
    for (int q = 0; q < 3; q++)
        if (outs[q] && !direct[q]) par_memcpy(outs[q], s->h_xfer + 3 * q * count, 3 * count * 8);
    if (T) mass_times(s, idx, count, T);
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_get_state(titan_gb300_sim *s, double *pos, double *vel, double *acc, double *T) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    return titan_gb300_get_masses(s, s->n, nullptr, pos, vel, acc, T);
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_mass_state(titan_gb300_sim *s, int64_t count, const int64_t *idx, const double *pos,
                               const double *vel, const double *m, const double *ext, const uint8_t *fixed,
                               const double *drag, const double *T) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (!idx) count = s->n;
    if (count < 0 || count > s->n) return s->fail(TITAN_GB300_EINVAL, "bad count");
    for (int64_t q = 0; idx && q < count; q++)
        if (idx[q] < 0 || idx[q] >= s->n) return s->fail(TITAN_GB300_EINVAL, "mass index out of range");
    if (m)
        for (int64_t q = 0; q < count; q++)
            if (!(m[q] > 0)) return s->fail(TITAN_GB300_EINVAL, "mass must be positive");
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    CK(cudaStreamSynchronize(s->stream), "set");
    bool replan = false;
    if (fixed) {
        if (s->fixed.empty()) s->fixed.assign(s->n, 0);
        for (int64_t q = 0; q < count; q++) {
            int64_t i = idx ? idx[q] : q;
            if ((s->fixed[i] != 0) != (fixed[q] != 0)) replan = true;
        }
    }
    // local time bookkeeping: masses whose T is given, or whose fixed flag
    // flips, restart their clock here
    std::vector<double> Tcur;
    if (replan || T) {
        Tcur.resize(s->n);
        mass_times(s, nullptr, s->n, Tcur.data());
    }
    // per-mass host bookkeeping, only for the attributes given (a loop over
    // every mass costs milliseconds on a million-mass scene)
    for (int64_t q = 0; (m || ext || drag || T || fixed) && q < count; q++) {
        int64_t i = idx ? idx[q] : q;
        if (m) s->m[i] = m[q];
        if (ext) {
            if (s->ext.empty()) s->ext.assign(3 * s->n, 0.0);
            for (int c = 0; c < 3; c++) s->ext[3 * i + c] = ext[3 * q + c];
        }
        if (drag) {
            if (s->drag.empty()) s->drag.assign(s->n, 0);
            s->drag[i] = (int32_t)drag[q];
        }
        if (T || (fixed && (s->fixed[i] != 0) != (fixed[q] != 0))) {
            s->mT0[i] = T ? T[q] : Tcur[i];
            s->mTstep[i] = s->steps;
        }
        if (fixed) s->fixed[i] = fixed[q] ? 1 : 0;
    }
    if (replan) {
        int rc = pull_state(s);
        if (rc) return rc;
        for (int64_t q = 0; q < count; q++) {
            int64_t i = idx ? idx[q] : q;
            for (int c = 0; c < 3; c++) {
                if (pos) s->pos[3 * i + c] = pos[3 * q + c];
                if (vel) s->vel[3 * i + c] = vel[3 * q + c];
            }
        }
        s->drop_graphs();
        return build_device(s);
    }
    if (m || ext || drag) {
        int rc = upload_mass_attrs(s);
        if (rc) return rc;
    }
    if (pos || vel) {
        tg::XferArgs x{};
        x.old2new = s->d_old2new;
        x.count = count;
        x.npad = s->npad;
        x.state0 = s->args.state0;
        x.state1 = s->args.state1;
        x.acc = s->args.acc;
        x.parity = s->parity;
        if (idx) {
            CK(cudaMemcpyAsync(s->d_idx, idx, count * 8, cudaMemcpyHostToDevice, s->stream), "upload index");
            x.idx = s->d_idx;
        }
        // a pinned caller buffer goes up by DMA directly, else through the
        // handle's pinned staging buffer
        const double *ins[2] = {pos, vel};
        for (int q = 0; q < 2; q++) {
            if (!ins[q]) continue;
            const double *src = ins[q];
            if (!host_pinned(src)) {
                par_memcpy(s->h_xfer + 3 * q * count, src, 3 * count * 8);
                src = s->h_xfer + 3 * q * count;
            }
            CK(cudaMemcpyAsync(s->d_xfer + 3 * q * count, src, 3 * count * 8, cudaMemcpyHostToDevice, s->stream),
               "upload");
        }
        x.ipos = pos ? s->d_xfer : nullptr;
        x.ivel = vel ? s->d_xfer + 3 * count : nullptr;
        CK(tg::launch_scatter(s->prec, x, s->stream), "scatter");
        CK(cudaStreamSynchronize(s->stream), "set");
    }
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

int titan_gb300_set_spring_params(titan_gb300_sim *s, int64_t count, const int64_t *idx, const double *k,
                                  const double *rest, const double *damping, const int32_t *type,
                                  const double *omega, const double *amp, const double *phase) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!idx) count = s->ns;
    if (count < 0 || count > s->ns) return s->fail(TITAN_GB300_EINVAL, "bad count");
    bool replan = false;
    for (int64_t q = 0; q < count; q++) {
        int64_t j = idx ? idx[q] : q;
        if (j < 0 || j >= s->ns) return s->fail(TITAN_GB300_EINVAL, "spring index out of range");
        if (type && (type[q] < 0 || type[q] > 3)) return s->fail(TITAN_GB300_EINVAL, "spring type must be 0..3");
    }
    for (int64_t q = 0; q < count; q++) {
        int64_t j = idx ? idx[q] : q;
        if (k) s->k[j] = k[q];
        if (rest) s->rest[j] = rest[q];
        if (damping) s->damping[j] = damping[q];
        if (type) {
            if (s->type.empty()) s->type.assign(s->ns, 0);
            bool was = s->type[j] >= 2, now = type[q] >= 2;
            if (was != now) replan = true;
            s->type[j] = type[q];
        }
        if (omega) {
            if (s->omega.empty()) s->omega.assign(s->ns, 0.0);
            s->omega[j] = omega[q];
        }
        if (amp) {
            if (s->amp.empty()) s->amp.assign(s->ns, 0.2);
            s->amp[j] = amp[q];
        }
        if (phase) {
            if (s->phase.empty()) s->phase.assign(s->ns, 0.0);
            s->phase[j] = phase[q];
        }
    }
    if (!s->started) return TITAN_GB300_OK;
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    CK(cudaStreamSynchronize(s->stream), "set springs");
    if (replan) {
        int rc = pull_state(s);
        if (rc) return rc;
        s->drop_graphs();
        return build_device(s);
    }
    // type changes within passive or within active keep the slab order, but
    // the type bits live in the entry words
    if (type) {
        for (size_t e = 0; e < s->plan.ent_ends.size(); e++) {
            int64_t j = s->plan.ent_spring[e];
            s->plan.ent_ends[e] = (s->plan.ent_ends[e] & 0x00ffffffu) | ((uint32_t)(s->type[j] & 3) << 24);
        }
        if (s->use_res)
            for (size_t q = 0; q < s->rplan.words.size(); q++) {
                int64_t j = s->rplan.rec_spring[q];
                if (j >= 0) s->rplan.words[q] = (s->rplan.words[q] & 0xffffu) | ((uint32_t)(s->type[j] & 3) << 16);
            }
    }
    return upload_entries(s);
} catch (...) {
    return host_exception(s);
}

int titan_gb300_diagnostics(titan_gb300_sim *s, double g_mag, double energy[4], double momentum[6]) try {
    if (!s) return TITAN_GB300_EINVAL;
    if (s->serving) return s->fail(TITAN_GB300_ESTATE, "the scene is being stepped by a request server");
    if (!s->started) return s->fail(TITAN_GB300_ESTATE, "The simulation has not started.");
    if (!ensure_device(s)) return s->fail(TITAN_GB300_ECUDA, "cudaSetDevice failed");
    cudaError_t e = cudaSuccess;
    if (!s->d_sl) {
        std::vector<int32_t> sl(s->ns, -1), sr(s->ns, -1);
        for (int64_t j = 0; j < s->ns; j++) {
            int32_t l = s->left[j], r = s->right[j];
            if (l < 0 || r < 0 || l >= s->n || r >= s->n) continue;
            sl[j] = s->plan.old2new[l];
            sr[j] = s->plan.old2new[r];
        }
        if (!(s->d_sl = dev_copy(s, sl, e))) return s->cuda_fail(e, "diag alloc");
        if (!(s->d_sr = dev_copy(s, sr, e))) return s->cuda_fail(e, "diag alloc");
        if (!(s->d_partials = (double *)s->mem.get(tg::kDiagBlocks * tg::kDiagQ * 8, e)))
            return s->cuda_fail(e, "diag alloc");
        if (!(s->d_dout = (double *)s->mem.get(tg::kDiagQ * 8, e))) return s->cuda_fail(e, "diag alloc");
        if (!(s->d_sk = (double *)s->mem.get(std::max<int64_t>(1, s->ns) * 8, e))) return s->cuda_fail(e, "diag alloc");
        if (!(s->d_srest = (double *)s->mem.get(std::max<int64_t>(1, s->ns) * 8, e)))
            return s->cuda_fail(e, "diag alloc");
    }
    if (s->ns > 0) {
        CK(cudaMemcpyAsync(s->d_sk, s->k.data(), s->ns * 8, cudaMemcpyHostToDevice, s->stream), "diag upload");
        CK(cudaMemcpyAsync(s->d_srest, s->rest.data(), s->ns * 8, cudaMemcpyHostToDevice, s->stream), "diag upload");
    }
    tg::DiagArgs d{};
    d.state = s->parity ? s->args.state1 : s->args.state0;
    d.mass = s->args.mass;
    d.n = s->n;
    d.npad = s->npad;
    d.sl = s->d_sl;
    d.sr = s->d_sr;
    d.sk = s->d_sk;
    d.srest = s->d_srest;
    d.ns = s->ns;
    d.g_mag = g_mag;
    d.partials = s->d_partials;
    d.out = s->d_dout;
    CK(tg::launch_diag(s->prec, d, s->stream), "diagnostics");
    double out[tg::kDiagQ];
    CK(cudaMemcpyAsync(out, s->d_dout, sizeof(out), cudaMemcpyDeviceToHost, s->stream), "diag download");
    CK(cudaStreamSynchronize(s->stream), "diagnostics");
    if (energy) {
        energy[0] = out[0];
        energy[1] = out[1];
        energy[2] = out[2];
        energy[3] = (out[0] + out[1]) + out[2];
    }
    if (momentum)
        for (int c = 0; c < 6; c++) momentum[c] = out[3 + c];
    return TITAN_GB300_OK;
} catch (...) {
    return host_exception(s);
}

void *titan_gb300_stream(titan_gb300_sim *s) { return s ? (void *)s->stream : nullptr; }

int titan_gb300_plan_info(const titan_gb300_sim *s, int64_t out[12]) {
    if (!s || !out) return TITAN_GB300_EINVAL;
    const tg::Plan &P = s->plan;
    std::memset(out, 0, 12 * sizeof(int64_t));
    out[0] = s->n;
    out[1] = s->ns;
    if (!s->started) return TITAN_GB300_OK;
    out[2] = P.ntiles;
    out[3] = (int64_t)P.ent_ends.size();
    out[4] = (int64_t)P.halo.size();
    out[5] = (int64_t)P.inc.size();
    out[6] = (int64_t)P.heavy_local.size();
    out[7] = (int64_t)s->smem;
    out[8] = s->threads;
    int64_t nact_springs = 0;
    if (!s->type.empty())
        for (int32_t t : s->type) nact_springs += t >= 2;
    int64_t nact_ent = 0;
    for (int32_t a : P.tile_nact) nact_ent += a;
    const bool f64 = s->prec == P_FP64;
    // algorithmic bytes per step: per mass read x,v,m,flags + write x,v;
    // per spring k, rest, damping + two endpoint indices; actuated springs
    // add omega and phase.
    int64_t mass_b = f64 ? 105 : (s->prec == P_FP32C ? 101 : 53);
    int64_t spring_b = f64 ? 32 : 20, act_b = f64 ? 16 : 8;
    out[9] = s->n * mass_b + P.valid_springs * spring_b + nact_springs * act_b;
    // implementation bytes as laid out: per mass state read (+halo re-reads)
    // and write, m, flags, degree; per entry record, act record, 2 B per
    // incidence word, 4 B per halo index, tile table.
    const int64_t rs = (int64_t)s->rsize();
    const int64_t comps = s->comps();
    int64_t impl = s->n * (comps * rs * 2 + rs + 1 + 1) + (int64_t)P.halo.size() * (f64 ? 48 : 36);
    impl += (int64_t)P.ent_ends.size() * (f64 ? 32 : 16) + nact_ent * (f64 ? 32 : 16);
    impl += (int64_t)P.inc.size() * 2 + (int64_t)P.heavy_inc.size() * 2 + (int64_t)P.halo.size() * 4;
    impl += P.ntiles * (int64_t)sizeof(tg::TileInfo);
    out[10] = s->use_pull ? s->pull_impl_bytes : impl;
    out[11] = nact_ent;
    return TITAN_GB300_OK;
}

int64_t titan_gb300_lattice_springs(int nx, int ny, int nz);

}  // extern "C"
