// engine.h -- device-side layout shared by the step kernels and the C ABI.
//
// HBM layout (all arrays in the tiled mass order of plan.h):
//   state[2]   ping-pong buffers of per-mass records (state.cuh):
//              FP64  48 B: x0 x1 | x2 v0 | v1 v2               (double)
//              FP32C 48 B: xh0 xh1 xh2 vh0 | vh1 vh2 xl0 xl1 | xl2 vl0 vl1 vl2
//                          (float hi/lo pairs)
//              FP32  32 B: x0 x1 x2 v0 | v1 v2 - -             (float)
//   mass, flags  per-mass m and MF_* bits; ext/lc/drag are only read for
//              masses whose flag asks for them; acc component-major (npad).
//   tiles      one TileInfo per tile.
//   ent        slab entries: FP64 {k, rest, damping, ends} (32 B),
//              FP32 {ends, k, rest, damping} (16 B); act parallel:
//              FP64 {omega, amp, phase, -}, FP32 {omega/2pi, +-amp, phase/2pi, -}.
//   inc        per-warp ELL incidence (u16 entry index, 0x8000 = left end),
//              4 codes per 8-byte word.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include <string>

#include "pull_layout.h"
#include "titan_gb300.h"

namespace tg {

enum { P_FP64 = 0, P_FP32 = 1, P_FP32C = 2 };
enum { MF_FIXED = 1, MF_EXT = 2, MF_LOCAL = 4, MF_DRAG = 8, MF_BODYPLANE = 16 };

constexpr int kMaxPlanes = 16;
constexpr int kMaxBalls = 16;

struct TileInfo {
    int32_t mass_off, nm, halo_off, nh;
    int32_t ent_off, ne, nact, warp_off;
    int32_t heavy_off, nheavy, body, inc_off;  // inc_off: first u16 word of the tile's incidence block
    int32_t inc_words, pad0, pad1, pad2;       // inc_words: length of that block (multiple of 128)
};

// Shared-memory layout of the warp-specialised persistent kernel
// (step_ws.cu): nstages stages, each [state records | slab records / force
// slots | actuation records | incidence block], the two-entry halo-index
// ring, the heavy-mass sums, the TileInfo of each stage, a copy of the
// DevParams, then 2 * nstages + 2 mbarriers and the control words.
struct WsLayout {
    int32_t slots, act, inc, stage, nstages;  // offsets inside a stage, stage size
    int32_t idx, idx_words;                   // halo-index ring (2 entries of idx_words int32)
    int32_t heavy, heavy_cap;                 // heavy sums: 2 groups x 3 x heavy_cap
    int32_t tinfo, params, mbar, total;       // per-stage TileInfo, DevParams copy, barriers
};
constexpr int kWsMaxStages = 3;
constexpr int kWsMaxConsumerWarps = 14;  // two groups of 7
constexpr int kWsProducerWarps = 2;      // share each tile's halo gathers: 512 threads in all

// Shared-memory layout of the pull kernel (step_pull.cu): nstages stages of
// one tile's state records (tile masses, then halo) and its actuation
// records (at act_off), the two-entry halo-index ring, a copy of the
// DevParams, 2 * nstages + 2 mbarriers and the control words.  Consumer
// warps form nteams teams of team_warps warps (one warp per 32 tile
// masses); team q takes the CTA's tiles q, q + nteams, ... in stages
// k % nstages (nstages a multiple of nteams).
struct PullLayout {
    int32_t stage, act_off, nstages, nteams, team_warps;
    int32_t idx, idx_words;        // halo-index ring (2 entries of idx_words int32)
    int32_t params, mbar, total;
};
constexpr int kPullMaxStages = 12;
constexpr int kPullMaxConsumerWarps = 15;  // + the producer warp: 512 threads (4 warps per SM sub-partition)

enum { INTEG_EULER = 0, INTEG_VERLET = 1, INTEG_RK2 = 2 };

struct DevParams {
    double dt;
    double g[3];
    int32_t nplanes, nballs;
    double plane[kMaxPlanes][6];  // normal xyz, offset, friction_k, friction_s
    double ball[kMaxBalls][4];    // center xyz, radius
    float dt_hi, dt_lo;
    float gf[3];
    float pad;
    float planef[kMaxPlanes][6];
    float ballf[kMaxBalls][4];
    int32_t integrator;           // INTEG_*
    float dt2f;                   // (float) pow(dt, 2)
    double dt2;                   // pow(dt, 2), computed on the host as the reference's Vec code does
    double launch_dt;             // time advanced by one launch: dt, or dt / 2 for RK2
    double pad2;
};

static_assert(sizeof(DevParams) % 16 == 0, "DevParams is copied as 16-byte vectors");

struct StepArgs {
    const TileInfo *tiles;
    const int32_t *halo;
    const void *ent;
    const void *act;
    const uint32_t *warp_inc_off;
    const uint8_t *deg;
    const uint16_t *inc;
    const uint16_t *heavy_local;
    const uint32_t *heavy_inc_off;
    const uint16_t *heavy_inc;
    const void *mass;
    const uint8_t *flags;
    const void *ext;           // 3 * npad, component-major
    const int32_t *lc_ptr;     // npad + 1
    const int32_t *lc_type;
    const double *lc_rec;      // 4 per record: vec xyz, num
    const int32_t *drag;
    const double *body_plane;  // 6 per body
    const float *body_planef;  // same, single precision
    void *state0;
    void *state1;
    void *acc;                 // 3 * npad
    double *tbuf;              // [2]: T of the step with parity p is tbuf[p]
    const DevParams *prm;
    int64_t npad;
    int32_t slots, ecap, hcap;
    int32_t ntiles;
    int32_t rk2_stage;         // RK2: 0 first half step, 1 second (launches alternate)
    int *err;                  // set by a kernel whose bounded wait gave up
    WsLayout ws;
    // pull form: unit descriptors (pull.team_warps slots per tile) and
    // their quad blocks (pull_layout.h)
    const PullUnit *pull_units;
    const uint8_t *pull_ell;
    PullLayout pull;
};

// Body-resident batched launch (resident.cu, plan.h ResPlan): bins of whole
// bodies, each run by one CTA for all steps of a launch with its state in
// shared memory.  Records use the slab-entry layout (entry_record_bytes)
// with the entry word replaced by the resident word.
struct ResArgs {
    const int64_t *bin_mass_off;   // nbins+1
    const int64_t *bin_warp_off;   // nbins+1
    const int32_t *mass;           // tiled index per resident mass
    const int32_t *body;
    const uint8_t *deg;
    const uint64_t *act_mask;
    const uint32_t *warp_rec_off;
    const void *rec;
    const void *act;
    int *next;                     // bin queue counter, zero at launch
    int64_t nbins;
    int32_t cap;                   // masses per bin (shared memory holds 2 * cap records)
};

// Resident tiles (resident_tiles.cu): tiles with no halo (every spring of
// their masses has both ends in the tile: a whole body, or a part of one
// that no spring joins to the rest) stepped by one CTA each for all steps
// of a launch, with the per-step kernels' two phases in shared memory.
struct TileResArgs {
    const TileInfo *tiles;  // the resident tiles
    const double *t0;       // T of the launch's first step (a copy taken before per-step kernels run beside it)
    int32_t ntiles;
    int32_t stage;          // 1: slab, actuation and incidence records staged in shared memory once per launch
};

// Per-mass gather / scatter between caller order and tiled order.
struct XferArgs {
    const int32_t *old2new;
    const int64_t *idx;        // caller indices, or null for 0..count-1
    int64_t count;
    int64_t npad;
    void *state0;
    void *state1;
    void *acc;
    int parity;
    double *pos, *vel, *accout;  // gather outputs (3*count), any may be null
    const double *ipos, *ivel;   // scatter inputs (3*count), any may be null
};

struct DiagArgs {
    const void *state;
    const void *mass;
    int64_t n, npad;
    const int32_t *sl, *sr;     // springs (new numbering), -1 = skipped
    const double *sk, *srest;
    int64_t ns;
    double g_mag;
    double *partials;           // kDiagBlocks * kDiagQ
    double *out;                // kDiagQ
};
constexpr int kDiagBlocks = 512;
constexpr int kDiagQ = 9;

// Raises kernel f's dynamic shared-memory limit on the current device to at
// least smem bytes, never lowering it: several engine handles in one process
// share the kernels, and a handle that needs less must not shrink the limit
// another handle's launches rely on.
cudaError_t raise_smem_limit(const void *f, size_t smem);

// words (of the precision's scalar) in one mass's state record
int state_words(int precision);
// dynamic shared memory of one tile's CTA
size_t tile_smem_bytes(int precision, int slots, int entries, int heavy);
// Per-tile kernel, launch-bound variant 0: (512 threads, 1 CTA/SM), every
// precision; FP32 forms also 1: (256, 3) and 2: (256, 4) -- at most 256
// threads per CTA, registers capped for 3 or 4 resident CTAs per SM.
constexpr int kStepVariants = 3;
const void *step_kernel_capped(int precision, int variant);  // null if not compiled
cudaError_t step_prepare(int precision, int variant, int integ, size_t smem);
cudaError_t launch_step(int precision, int variant, int integ, const StepArgs &a, int ntiles, int threads,
                        size_t smem, int parity, int write_acc, cudaStream_t s);
// Per-tile kernel with asynchronous staging (step_async.cu): slab records and
// tile states by bulk copy, halo by cp.async, one wait.  Shared memory per
// CTA: tile_async_smem_bytes.
size_t tile_async_smem_bytes(int precision, int slots, int entries, int heavy);
cudaError_t step_async_prepare(int precision, size_t smem);
cudaError_t launch_step_async(int precision, const StepArgs &a, int ntiles, int threads, size_t smem, int parity,
                              int write_acc, cudaStream_t s);
// Warp-specialised persistent kernel (step_ws.cu): `ctas` CTAs of
// consumer_warps + 1 warps; the last warp streams tiles into a ring of
// stages, the others compute.
cudaError_t step_ws_prepare(int precision, int integ, size_t smem);
cudaError_t launch_step_ws(int precision, int integ, const StepArgs &a, int ctas, int consumer_warps, int parity,
                           int write_acc, cudaStream_t s);
// Pull kernel (step_pull.cu): `ctas` persistent CTAs of a.pull's teams
// plus a producer warp; FP32 and FP32C only.
cudaError_t step_pull_prepare(int precision, int integ, size_t smem);
cudaError_t launch_step_pull(int precision, int integ, const StepArgs &a, int ctas, int parity, int write_acc,
                             cudaStream_t s);
// bytes of one state record / one slab entry record for a precision
int state_record_bytes(int precision);
int entry_record_bytes(int precision);
// Resident launch: `nsteps` steps of every bin, starting from parity;
// masses per thread = ceil(cap / threads) must be at most kResMaxMpt.
constexpr int kResMaxMpt = 4;
size_t resident_smem_bytes(int precision, int cap);
cudaError_t resident_prepare(int precision, int mpt, size_t smem);
int resident_ctas_per_sm(int precision, int mpt, int threads, size_t smem);
cudaError_t launch_resident(int precision, const StepArgs &a, const ResArgs &r, int ctas, int threads, int parity,
                            int64_t nsteps, int write_acc, int write_time, cudaStream_t s);
// The device time record advanced by nsteps additions of dt, for launches
// with no per-step tiles.
cudaError_t launch_advance_time(const StepArgs &a, int parity, int64_t nsteps, cudaStream_t s);
// Resident tiles: shared memory of one tile (state twice, force slots and
// the zero slot, heavy sums, and with stage the tile's slab, actuation and
// incidence records; launch parameters first), and the launch (masses per
// thread = ceil(largest tile / threads) at most kResMaxMpt).
size_t tile_resident_smem_bytes(int precision, const TileInfo &ti, int stage);
cudaError_t tile_resident_prepare(int precision, int mpt, int stage, size_t smem);
int tile_resident_ctas_per_sm(int precision, int mpt, int stage, int threads, size_t smem);
cudaError_t launch_tile_resident(int precision, const StepArgs &a, const TileResArgs &r, int mpt, int threads,
                                 size_t smem, int parity, int64_t nsteps, int write_acc, cudaStream_t s);
cudaError_t launch_gather(int precision, const XferArgs &a, cudaStream_t s);
// float positions of all a.count masses in caller order into out (device)
cudaError_t launch_export_f32(int precision, const XferArgs &a, float *out, cudaStream_t s);
cudaError_t launch_scatter(int precision, const XferArgs &a, cudaStream_t s);
cudaError_t launch_diag(int precision, const DiagArgs &a, cudaStream_t s);

// A started scene handed to the request server (server.cu): its step
// arguments and step parity.  serve_begin checks that the server can step
// it (same device and precision, symplectic Euler, every tile on the
// per-step kernels, tiles within tile_smem bytes of shared memory), waits for
// the scene's own queued work and marks it busy (its own stepping, transfers
// and parameter changes are refused until serve_end); serve_end advances the
// scene's host-side clock and step count by nsteps (nsteps < 0: abandoned,
// the scene's state is then undefined) and releases it.
struct ServeScene {
    const StepArgs *args;
    int parity;
};
int serve_begin(titan_gb300_sim *s, int device, int precision, size_t tile_smem, ServeScene &v, std::string &why);
void serve_end(titan_gb300_sim *s, int64_t nsteps);

}  // namespace tg
