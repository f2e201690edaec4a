// plan.cpp -- builds the tile plan described in plan.h.
#include "plan.h"

#include <algorithm>
#include <cmath>
#include <deque>
#include <numeric>
#include <utility>

namespace tg {

namespace {

// Interleave the low 21 bits of v with two zero bits between each.
uint64_t spread21(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

bool actuated(const PlanInput &in, int64_t s) {
    return in.type && (in.type[s] == 2 || in.type[s] == 3);
}

}  // namespace

std::string build_plan(const PlanInput &in, Plan &P) {
    P = Plan();
    const int64_t n = in.n, ns = in.ns;
    P.n = n;
    P.ns = ns;
    if (n <= 0) return "no masses";
    if (n >= (int64_t(1) << 31) - 1) return "more than 2^31-2 masses";
    if (in.tile_cap < 32 || in.tile_cap > 2048) return "tile size must be in [32, 2048]";
    if (in.heavy_threshold < 1 || in.heavy_threshold > 254) return "heavy threshold must be in [1, 254]";

    // ---- bodies --------------------------------------------------------
    std::vector<int64_t> bptr;
    if (in.nbodies > 0 && in.body_ptr) {
        bptr.assign(in.body_ptr, in.body_ptr + in.nbodies + 1);
        if (bptr.front() != 0 || bptr.back() != n) return "body ranges must cover all masses";
        for (int64_t b = 0; b < in.nbodies; b++)
            if (bptr[b + 1] <= bptr[b]) return "body ranges must be non-empty and increasing";
    } else {
        bptr = {0, n};
    }
    P.nbodies = (int64_t)bptr.size() - 1;

    // ---- spatial order inside each body (Morton code of the start pose) --
    P.new2old.resize(n);
    std::iota(P.new2old.begin(), P.new2old.end(), 0);
    std::vector<uint64_t> code(n, 0);
    for (int64_t b = 0; b < P.nbodies; b++) {
        int64_t b0 = bptr[b], b1 = bptr[b + 1];
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t i = b0; i < b1; i++)
            for (int c = 0; c < 3; c++) {
                double x = in.pos[3 * i + c];
                if (std::isfinite(x)) {
                    lo[c] = std::min(lo[c], x);
                    hi[c] = std::max(hi[c], x);
                }
            }
        double span = 0;
        for (int c = 0; c < 3; c++)
            if (hi[c] > lo[c]) span = std::max(span, hi[c] - lo[c]);
        double scale = span > 0 ? 2097151.0 / span : 0.0;
        for (int64_t i = b0; i < b1; i++) {
            uint64_t q[3];
            for (int c = 0; c < 3; c++) {
                double x = in.pos[3 * i + c];
                double t = std::isfinite(x) && lo[c] <= hi[c] ? (x - lo[c]) * scale : 0.0;
                t = std::min(std::max(t, 0.0), 2097151.0);
                q[c] = (uint64_t)t;
            }
            code[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
        }
        std::stable_sort(P.new2old.begin() + b0, P.new2old.begin() + b1,
                         [&](int32_t a, int32_t c) { return code[a] < code[c]; });
    }
    P.old2new.resize(n);
    for (int64_t i = 0; i < n; i++) P.old2new[P.new2old[i]] = (int32_t)i;

    // ---- springs in the new numbering -----------------------------------
    std::vector<int32_t> L(ns, -1), R(ns, -1);
    for (int64_t s = 0; s < ns; s++) {
        int32_t l = in.left[s], r = in.right[s];
        if (l < 0 || r < 0 || l >= n || r >= n) continue;  // skipped as src/sim.cu:1052 does
        L[s] = P.old2new[l];
        R[s] = P.old2new[r];
        P.valid_springs++;
    }
    auto is_fixed_new = [&](int64_t m) { return in.fixed && in.fixed[P.new2old[m]]; };

    // incidence of each (non-fixed) mass, ascending spring order; for a spring
    // attached twice to one mass the right end comes first (src/sim.cu:1067-1077)
    std::vector<int64_t> ip(n + 1, 0);
    for (int64_t s = 0; s < ns; s++) {
        if (L[s] < 0) continue;
        if (!is_fixed_new(R[s])) ip[R[s] + 1]++;
        if (!is_fixed_new(L[s])) ip[L[s] + 1]++;
    }
    for (int64_t i = 0; i < n; i++) ip[i + 1] += ip[i];
    std::vector<int64_t> isp(ip[n]);
    std::vector<int8_t> isg(ip[n]);
    {
        std::vector<int64_t> fill(ip.begin(), ip.end() - 1);
        for (int64_t s = 0; s < ns; s++) {
            if (L[s] < 0) continue;
            if (!is_fixed_new(R[s])) { isp[fill[R[s]]] = s; isg[fill[R[s]]] = 1; fill[R[s]]++; }
            if (!is_fixed_new(L[s])) { isp[fill[L[s]]] = s; isg[fill[L[s]]] = -1; fill[L[s]]++; }
        }
    }

    // ---- tiles ------------------------------------------------------------
    std::vector<int64_t> smark(ns, -1);
    std::vector<int32_t> elocal(ns, 0);
    std::vector<int64_t> hmark(n, -1);
    std::vector<int32_t> hslot(n, 0);
    std::vector<int64_t> ents, ents_act;
    std::vector<int32_t> halo;
    int64_t attempt = 0;

    P.tile_mass_off.push_back(0);
    P.tile_halo_off.push_back(0);
    P.tile_ent_off.push_back(0);
    P.tile_warp_off.push_back(0);
    P.tile_heavy_off.push_back(0);
    P.deg.assign(n, 0);

    for (int64_t b = 0; b < P.nbodies; b++) {
        std::deque<std::pair<int64_t, int64_t>> work;
        for (int64_t lo = bptr[b]; lo < bptr[b + 1]; lo += in.tile_cap)
            work.emplace_back(lo, std::min(lo + (int64_t)in.tile_cap, bptr[b + 1]));
        while (!work.empty()) {
            auto [lo, hi] = work.front();
            work.pop_front();
            const int64_t nm = hi - lo;
            attempt++;
            ents.clear();
            ents_act.clear();
            halo.clear();
            for (int64_t m = lo; m < hi; m++)
                for (int64_t q = ip[m]; q < ip[m + 1]; q++) {
                    int64_t s = isp[q];
                    if (smark[s] == attempt) continue;
                    smark[s] = attempt;
                    (actuated(in, s) ? ents_act : ents).push_back(s);
                }
            int64_t ne = (int64_t)(ents.size() + ents_act.size());
            bool fits = ne <= in.entry_cap;
            if (fits) {
                for (auto *v : {&ents_act, &ents})
                    for (int64_t s : *v)
                        for (int32_t x : {L[s], R[s]})
                            if ((x < lo || x >= hi) && hmark[x] != attempt) {
                                hmark[x] = attempt;
                                halo.push_back(x);
                            }
                fits = nm + (int64_t)halo.size() <= in.slot_cap;
                if (fits) {
                    int64_t heavy = 0;
                    for (int64_t m = lo; m < hi; m++) heavy += (ip[m + 1] - ip[m]) > in.heavy_threshold;
                    fits = (nm + (int64_t)halo.size()) * in.slot_bytes + ne * in.entry_bytes +
                               heavy * in.heavy_bytes <= in.smem_budget;
                }
            }
            if (!fits) {
                if (nm == 1)
                    return "mass " + std::to_string(P.new2old[lo]) + " has " +
                           std::to_string(ip[lo + 1] - ip[lo]) +
                           " springs, more than one tile's slab can hold";
                int64_t mid = lo + nm / 2;
                work.emplace_front(mid, hi);
                work.emplace_front(lo, mid);
                continue;
            }
            // commit tile
            std::sort(ents_act.begin(), ents_act.end());
            std::sort(ents.begin(), ents.end());
            std::sort(halo.begin(), halo.end());
            const int64_t nh = (int64_t)halo.size();
            for (int64_t i = 0; i < nh; i++) hslot[halo[i]] = (int32_t)(nm + i);
            auto slot = [&](int32_t x) -> uint32_t {
                return (x >= lo && x < hi) ? (uint32_t)(x - lo) : (uint32_t)hslot[x];
            };
            int32_t e = 0;
            for (auto *v : {&ents_act, &ents})
                for (int64_t s : *v) {
                    elocal[s] = e++;
                    P.ent_ends.push_back(pack_ends(slot(L[s]), slot(R[s]), in.type ? (uint32_t)in.type[s] : 0u));
                    P.ent_spring.push_back(s);
                }
            P.halo.insert(P.halo.end(), halo.begin(), halo.end());
            while (P.halo.size() % 4) P.halo.push_back(halo.empty() ? (int32_t)lo : halo.back());
            P.tile_nh.push_back((int32_t)nh);
            P.tile_nact.push_back((int32_t)ents_act.size());

            int nheavy = 0;
            const int64_t nwarps = (nm + 31) / 32;
            for (int64_t w = 0; w < nwarps; w++) {
                int64_t m0 = lo + 32 * w, m1 = std::min(m0 + 32, hi);
                int64_t width = 0;
                for (int64_t m = m0; m < m1; m++) {
                    int64_t d = ip[m + 1] - ip[m];
                    if (d <= in.heavy_threshold) width = std::max(width, d);
                }
                width = (width + 3) & ~int64_t(3);
                if (P.inc.size() > 0xffffffffULL - (uint64_t)(width * 32))
                    return "incidence table exceeds 2^32 words";
                uint32_t off = (uint32_t)P.inc.size();
                P.warp_inc_off.push_back(off);
                P.inc.resize(P.inc.size() + (size_t)(width * 32), 0);
                for (int64_t m = m0; m < m1; m++) {
                    int64_t d = ip[m + 1] - ip[m];
                    int64_t lane = m - m0;
                    auto code_of = [&](int64_t q) -> uint16_t {
                        return (uint16_t)(elocal[isp[q]] | (isg[q] < 0 ? 0x8000 : 0));
                    };
                    if (d <= in.heavy_threshold) {
                        P.deg[m] = (uint8_t)d;
                        for (int64_t j = 0; j < d; j++)
                            P.inc[ell_index(off, (uint32_t)lane, (uint32_t)j)] = code_of(ip[m] + j);
                    } else {
                        P.deg[m] = 255;
                        P.heavy_local.push_back((uint16_t)(m - lo));
                        P.heavy_inc_off.push_back((uint32_t)P.heavy_inc.size());
                        for (int64_t q = ip[m]; q < ip[m + 1]; q++) P.heavy_inc.push_back(code_of(q));
                        nheavy++;
                    }
                }
            }
            P.body_of_tile.push_back((int32_t)b);
            P.tile_mass_off.push_back(hi);
            P.tile_halo_off.push_back((int64_t)P.halo.size());
            P.tile_ent_off.push_back((int64_t)P.ent_ends.size());
            P.tile_warp_off.push_back(P.tile_warp_off.back() + nwarps);
            P.tile_heavy_off.push_back((int64_t)P.heavy_local.size());
            P.max_nm = std::max<int>(P.max_nm, (int)nm);
            P.max_slots = std::max<int>(P.max_slots, (int)(nm + nh));
            P.max_entries = std::max<int>(P.max_entries, (int)ne);
            P.max_heavy = std::max(P.max_heavy, nheavy);
        }
    }
    P.heavy_inc_off.push_back((uint32_t)P.heavy_inc.size());
    P.ntiles = (int64_t)P.body_of_tile.size();
    return "";
}

}  // namespace tg
