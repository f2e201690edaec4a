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
// 32 u + l), built from the tile plan.  Every tile has team_warps unit slots
// (unit u of tile t is units[t * team_warps + u]; slots past the tile's
// masses have lanes == 0), so a warp finds its next unit without reading the
// tile record first.  A unit's columns (lane l's j-th spring in its
// incidence order) come in quads of four columns, each quad a 128-byte
// aligned block of
//     words    uint16 [32 lanes][4]  neighbour's state record as a float4
//                                    index (tile-local slot * record
//                                    float4s) | PW_VALID | PW_ACT
//     k        float  [32][4]
//     rest     float  [32][4]        for an actuated spring: the bits of its
//                                    slab entry index (< the tile's nact),
//                                    whose actuation record {nu, +-amp, phi,
//                                    rest} the producer stages with the
//                                    tile's states
//     damping  float  [32][4]        only when PU_DAMP (else the unit's
//                                    uniform PullUnit::damping)
// Columns past a lane's degree are padding (word 0).
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
    uint32_t ell;     // first quad, in 128-byte units
    uint16_t nquads;  // quads of columns (the unit's largest degree, rounded up to 4, / 4)
    uint8_t lanes;    // masses in the unit (0: no unit in this slot)
    uint8_t flags;    // PU_DAMP: per-column damping
    float damping;    // the unit's damping when uniform
    int32_t mass0;    // tiled index of lane 0's mass
};
static_assert(sizeof(PullUnit) == 16, "PullUnit is loaded as one 16-byte vector");

enum { PU_DAMP = 1 };
enum : uint32_t { PW_VALID = 0x4000u, PW_ACT = 0x8000u, PW_SLOT = 0x3fffu };

// bytes of one quad block
TG_PULL_HD inline constexpr uint32_t pull_quad_bytes(bool damp) { return damp ? 1792u : 1280u; }

}  // namespace tg
