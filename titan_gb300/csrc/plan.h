// plan.h -- host-side tile plan for the fused step kernel.
//
// The reference launches one thread per spring that atomically adds its force
// into both endpoint masses (src/sim.cu:1046-1080, src/vec.cu:33-37), then one
// thread per mass (src/sim.cu:1093-1169).  Here masses are renumbered into
// spatially compact tiles; each tile owns a slab of spring entries (every
// spring touching the tile, stored once per tile it touches), a halo of
// remote masses those entries read, and per-mass incidence lists into the slab
// in ascending spring order.  One CTA per tile computes each slab entry once
// and gathers per mass in a fixed order: deterministic, no float atomics.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "pull_layout.h"

namespace tg {

struct PlanInput {
    int64_t n = 0;                       // masses
    const double *pos = nullptr;         // 3n, used for the spatial order
    const uint8_t *fixed = nullptr;      // n or null; fixed masses gather nothing
    int64_t ns = 0;                      // springs
    const int32_t *left = nullptr, *right = nullptr;
    const int32_t *type = nullptr;       // ns or null; types 2,3 are actuated
    int64_t nbodies = 0;                 // 0: one body
    const int64_t *body_ptr = nullptr;   // nbodies+1, creation-order ranges
    int tile_cap = 512;                  // masses per tile
    int whole_cap = 0;                   // bodies of at most this many masses stay one tile (0: tile_cap)
    int slot_cap = 4095;                 // tile + halo slots per tile (12-bit)
    int entry_cap = 32767;               // slab entries per tile (15-bit)
    int heavy_threshold = 96;            // degree above this: warp-cooperative
    // shared-memory budget of one tile: slots * slot_bytes + entries *
    // entry_bytes + heavy masses * heavy_bytes must not exceed smem_budget
    int64_t smem_budget = 1 << 30;
    int slot_bytes = 0, entry_bytes = 0, heavy_bytes = 0;
};

// Incidence words are stored four per lane: for the warp holding a mass at
// lane l, code j of that mass is inc[warp_off + (j / 4) * 128 + 4 * l + j % 4],
// so one 8-byte load fetches four codes and a warp's load is 256 contiguous
// bytes.  A warp's block width is its largest degree rounded up to 4.
inline uint64_t ell_index(uint64_t warp_off, uint32_t lane, uint32_t j) {
    return warp_off + (uint64_t)(j >> 2) * 128 + 4 * lane + (j & 3);
}

// Entry word: left slot | right slot << 12 | type << 24 (slots are tile-local:
// [0, nm) tile masses, [nm, nm+nh) halo masses).
inline uint32_t pack_ends(uint32_t a, uint32_t b, uint32_t type) {
    return a | (b << 12) | ((type & 3u) << 24);
}

struct Plan {
    int64_t n = 0, ns = 0, ntiles = 0, nbodies = 1;
    std::vector<int32_t> new2old, old2new;   // mass renumbering
    std::vector<int32_t> body_of_tile;
    std::vector<int64_t> tile_mass_off;      // ntiles+1 (new mass index)
    std::vector<int64_t> tile_halo_off;      // ntiles+1, multiples of 4 (16-byte aligned lists)
    std::vector<int32_t> tile_nh;            // halo masses of each tile (lists are padded to 4)
    std::vector<int32_t> halo;               // new mass indices
    std::vector<int64_t> tile_ent_off;       // ntiles+1
    std::vector<int32_t> tile_nact;          // actuated entries lead each slab
    std::vector<uint32_t> ent_ends;
    std::vector<int64_t> ent_spring;         // original spring index of each entry
    std::vector<int64_t> tile_warp_off;      // ntiles+1 (global warp index)
    std::vector<uint32_t> warp_inc_off;      // per warp, into inc (u16 words)
    std::vector<uint8_t> deg;                // per new mass; 255 = heavy
    std::vector<uint16_t> inc;               // entry | 0x8000 when the mass is the left end; padding: ne
    std::vector<int64_t> tile_heavy_off;     // ntiles+1 (global heavy index)
    std::vector<uint16_t> heavy_local;       // tile-local index of each heavy mass
    std::vector<uint32_t> heavy_inc_off;     // nheavy+1, into heavy_inc
    std::vector<uint16_t> heavy_inc;
    int64_t valid_springs = 0;
    int max_nm = 0, max_slots = 0, max_entries = 0, max_heavy = 0;
};

// Returns "" on success, otherwise the reason (e.g. a mass whose degree does
// not fit one tile's slab, or host memory exhausted); throws nothing.
std::string build_plan(const PlanInput &in, Plan &out);

// Body-resident plan: bodies small enough for one CTA keep their state in
// shared memory for a whole multi-step launch.  Whole bodies are packed into
// bins of at most bin_cap masses (best fit, largest body first); one CTA
// runs one bin at a time.  Each bin-local mass lists its springs in
// ascending order as records whose word is
//   other end's bin-local index | 0x8000 if this mass is the right end |
//   type << 16
// laid out per warp of 32 bin-local masses as ELL: record j of lane l of
// bin warp w is warp_rec_off[w] + 32 j + l.
struct ResPlan {
    int64_t nbins = 0;
    int bin_cap = 0;
    std::vector<int64_t> bin_mass_off;   // nbins+1, into the per-resident-mass arrays
    std::vector<int64_t> bin_warp_off;   // nbins+1, into warp_rec_off
    std::vector<int32_t> mass;           // tiled index of each resident mass (bin order)
    std::vector<int32_t> body;           // its body
    std::vector<uint8_t> deg;            // its degree (free masses; 0 if fixed)
    std::vector<uint64_t> act_mask;      // bit j: record j (j < 64) is actuated
    std::vector<uint32_t> warp_rec_off;  // first record of each bin warp
    std::vector<uint32_t> words;         // one per record (padding: 0)
    std::vector<int64_t> rec_spring;     // spring of each record, -1 = padding
    std::vector<uint8_t> resident;       // per body: 1 if resident
    std::vector<uint8_t> tile_resident;  // per tile of Plan: 1 if it belongs to a resident body
    int64_t nmasses = 0, nbodies = 0;
};

// Picks the bodies with at most max_masses masses, no mass of degree above
// 254 (free masses only count) and no spring to another body, and packs
// them into bins of bin_cap masses (bin_cap >= max_masses).
void build_resident(const PlanInput &in, const Plan &P, int max_masses, int bin_cap, ResPlan &R);

// Spring tables of the pull form (pull_layout.h), derived from a tile plan
// for the tiles the per-step kernel runs: team_warps unit slots per tile;
// lane l of unit u lists the springs of tile mass 32u + l in its incidence
// order (ascending spring index), each as the other end's state record
// (float4 index: tile-local slot * rec_f4) and the spring's k, rest and
// damping in the FP32 forms' rounding; an actuated spring carries its slab
// entry index in place of rest.
struct PullTile {
    int64_t mass_off = 0, ent_off = 0, warp_off = 0;
    int32_t nm = 0;
};
struct PullSprings {
    const double *k = nullptr, *rest = nullptr, *damping = nullptr;
};
struct PullTables {
    int team_warps = 0;
    std::vector<PullUnit> units;  // ntiles * team_warps
    std::vector<uint8_t> ell;     // quad blocks
};
// Returns "" on success, else why the pull form cannot run the plan (a heavy
// mass, whose incidence list the plan keeps apart); throws nothing.
std::string build_pull(const Plan &P, const std::vector<PullTile> &tiles, int team_warps, int rec_f4,
                       const PullSprings &sp, PullTables &out);

}  // namespace tg
