// pull_layout.h -- spring tables of the pull form of the step (step_pull.cu).
//
// In the pull form every mass computes the forces of its own springs, each
// spring once at each end, from the state records its tile stages in shared
// memory, and sums them in its incidence order (ascending spring index).
// The force of a spring computed at either end is the same value up to sign
// (d = x_r - x_l changes sign exactly, |d|, the damping term and the scale
// do not), so the sums equal the slab forms' bit for bit.
//
// Tables, per unit of 32 consecutive tile masses (lane l = tile-local mass
// 32 u + l), built from the tile plan:
//   unit block (128-byte aligned, ncols = the unit's largest degree):
//     words    uint16 [ncols][32]  neighbour's tile-local slot | 0x8000 when
//                                  the spring is actuated (padded to 128 B)
//     k        float  [ncols][32]
//     rest     float  [ncols][32]
//     damping  float  [ncols][32]  read only when the unit's damping is not
//                                  uniform (PU_DAMP), else PullUnit::damping
//   column j of lane l is that mass's j-th spring; lanes whose degree is at
//   most j have no column j (never read).
//   actuation block (16-byte records, at PullUnit::act): a header of
//     kPullActHeader records holding uint16 off[33] -- lane l's records are
//     [off[l], off[l+1]) after the header -- then records {nu = omega / 2 pi,
//     +-amp (minus for contract-then-expand), phi = phase / 2 pi, 0} in each
//     lane's incidence order.
#pragma once

#include <cstdint>

// the layout helpers are used by host code (the planner, compiled by the
// host compiler) and by the kernel
#if defined(__CUDACC__)
#define TG_PULL_HD __host__ __device__
#else
#define TG_PULL_HD
#endif

namespace tg {

struct PullUnit {
    uint32_t ell;     // unit block offset in 128-byte units
    uint16_t ncols;   // columns (largest degree among the unit's masses)
    uint16_t flags;   // PU_DAMP: per-column damping
    float damping;    // the unit's damping when uniform
    uint32_t act;     // actuation header offset in 16-byte records
};
static_assert(sizeof(PullUnit) == 16, "PullUnit is loaded as one 16-byte vector");

enum { PU_DAMP = 1 };
constexpr int kPullActHeader = 5;  // 33 uint16 lane offsets in 16-byte records

// bytes of the words array of a unit block with ncols columns
TG_PULL_HD inline constexpr uint32_t pull_words_bytes(int ncols) { return (uint32_t)((ncols * 64 + 127) & ~127); }
// bytes of a whole unit block
TG_PULL_HD inline constexpr uint64_t pull_block_bytes(int ncols) { return pull_words_bytes(ncols) + 3ull * (uint64_t)ncols * 128; }

}  // namespace tg
