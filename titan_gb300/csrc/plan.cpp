// plan.cpp -- builds the tile plan described in plan.h.
#include "plan.h"

#include <algorithm>
#include <system_error>
#include <thread>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <new>
#include <mutex>
#include <exception>
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

// Recursive coordinate bisection of ids[0, cnt) (mass indices, reordered
// in place) into ceil(cnt / cap) leaves; each leaf ends up in Morton order
// and its end (offset base + position) is appended to leaf_end.  Ties on
// the split axis are broken by Morton code, then index: a total order, so
// the leaves' contents do not depend on the selection algorithm.
// Host threads of the planner: TITAN_GB300_PLAN_THREADS when set (1 to
// 64), else the host's processors, at most 16.  The plan does not depend on it.
int planner_threads() {
    if (const char *e = std::getenv("TITAN_GB300_PLAN_THREADS")) {
        const int v = std::atoi(e);
        if (v >= 1) return std::min(v, 64);
    }
    return (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
}

// The two halves of a cut are independent: down to `par_depth` levels the
// second half runs on its own thread, its leaves appended after the first's.
void bisect(int32_t *ids, int64_t cnt, int cap, const std::vector<uint32_t> &qc, const std::vector<uint64_t> &code,
            int64_t base, std::vector<int64_t> &leaf_end, int par_depth = 0) {
    if (cnt <= 0) return;
    const int64_t m = (cnt + cap - 1) / cap;
    if (m <= 1) {
        std::sort(ids, ids + cnt, [&](int32_t a, int32_t c) { return code[a] < code[c] || (code[a] == code[c] && a < c); });
        leaf_end.push_back(base + cnt);
        return;
    }
    uint32_t lo[3] = {UINT32_MAX, UINT32_MAX, UINT32_MAX}, hi[3] = {0, 0, 0};
    for (int64_t q = 0; q < cnt; q++)
        for (int c = 0; c < 3; c++) {
            lo[c] = std::min(lo[c], qc[3 * (size_t)ids[q] + c]);
            hi[c] = std::max(hi[c], qc[3 * (size_t)ids[q] + c]);
        }
    int ax = 0;
    for (int c = 1; c < 3; c++)
        if (hi[c] - lo[c] > hi[ax] - lo[ax]) ax = c;
    const int64_t m1 = m / 2;
    const int64_t k = (int64_t)std::llround((double)cnt * (double)m1 / (double)m);
    std::nth_element(ids, ids + k, ids + cnt, [&](int32_t a, int32_t c) {
        const uint32_t xa = qc[3 * (size_t)a + ax], xc = qc[3 * (size_t)c + ax];
        return xa < xc || (xa == xc && (code[a] < code[c] || (code[a] == code[c] && a < c)));
    });
    if (par_depth > 0 && cnt >= (int64_t)1 << 15) {
        std::vector<int64_t> second;
        std::exception_ptr err;
        std::thread th;
        try {
            th = std::thread([&] {
                try {
                    bisect(ids + k, cnt - k, cap, qc, code, base + k, second, par_depth - 1);
                } catch (...) {
                    err = std::current_exception();
                }
            });
        } catch (const std::system_error &) {  // no thread to be had: both halves here
            bisect(ids, k, cap, qc, code, base, leaf_end, par_depth - 1);
            bisect(ids + k, cnt - k, cap, qc, code, base + k, leaf_end, par_depth - 1);
            return;
        }
        try {
            bisect(ids, k, cap, qc, code, base, leaf_end, par_depth - 1);
        } catch (...) {
            th.join();
            throw;
        }
        th.join();
        if (err) std::rethrow_exception(err);
        leaf_end.insert(leaf_end.end(), second.begin(), second.end());
        return;
    }
    bisect(ids, k, cap, qc, code, base, leaf_end);
    bisect(ids + k, cnt - k, cap, qc, code, base + k, leaf_end);
}

bool actuated(const PlanInput &in, int64_t s) {
    return in.type && (in.type[s] == 2 || in.type[s] == 3);
}


// Orders one part of a tile's slab (entries given with their left and right
// state-record slots) so that each aligned group of eight entries -- the
// eight lanes of one quarter-warp, whose 16-byte shared-memory loads of the
// endpoint records are served together -- reads its records from distinct
// bank groups where it can.  A 48-byte record at slot x puts its k-th
// 16-byte piece in bank group (3x + k) mod 8 and a 32-byte one in (2x + k)
// mod 8, so two entries of a group conflict when their left (or right) slots
// differ but agree mod 8 (48-byte records) or mod 4 (32-byte records; at
// most two distinct slots per residue are then unavoidable).  Equal slots
// are one broadcast and never conflict.  The part starts `lead` entries
// into a group whose earlier entries (the previous part's last ones) have
// slots lead_ls / lead_rs.  Greedy, in spring order: each group takes the
// first remaining entries within a window that add no conflict, then fills
// up with the first remaining ones.  The order of an entry in the slab
// changes no result: each mass sums its entries' forces in its incidence
// order.
void bank_order(std::vector<int64_t> &v, const std::vector<uint32_t> &ls, const std::vector<uint32_t> &rs,
                int record_bytes, const uint32_t *lead_ls, const uint32_t *lead_rs, int lead) {
    const int64_t n = (int64_t)v.size();
    const int mod = record_bytes == 32 ? 4 : 8, cap = 8 / mod;
    constexpr int kWindow = 64;
    // unused entries as a doubly linked list in spring order (n: the end)
    std::vector<int64_t> nx(n + 1), pv(n + 1);
    for (int64_t q = 0; q <= n; q++) {
        nx[q] = q + 1;
        pv[q] = q - 1;
    }
    int64_t head = n > 0 ? 0 : n;
    auto take = [&](int64_t q) {
        if (pv[q] >= 0) nx[pv[q]] = nx[q];
        else head = nx[q];
        if (nx[q] <= n) pv[nx[q]] = pv[q];
    };
    std::vector<int64_t> out;
    out.reserve(n);
    std::vector<uint8_t> lr(n), rr(n);  // residues of the endpoint slots
    for (int64_t q = 0; q < n; q++) {
        lr[q] = (uint8_t)(ls[q] % (uint32_t)mod);
        rr[q] = (uint8_t)(rs[q] % (uint32_t)mod);
    }
    bool first = true;
    while ((int64_t)out.size() < n) {
        uint32_t lsl[8][2], rsl[8][2];
        int lcnt[8] = {0}, rcnt[8] = {0};
        auto fits = [&](const uint32_t (*tab)[2], const int *cnt, uint32_t x, int r) {
            for (int q = 0; q < cnt[r]; q++)
                if (tab[r][q] == x) return true;
            return cnt[r] < cap;
        };
        auto add = [&](uint32_t (*tab)[2], int *cnt, uint32_t x) {
            const int r = (int)(x % (uint32_t)mod);
            for (int q = 0; q < cnt[r]; q++)
                if (tab[r][q] == x) return;
            if (cnt[r] < cap) tab[r][cnt[r]++] = x;
        };
        int taken = 0;
        if (first) {
            for (int q = 0; q < lead; q++) {
                add(lsl, lcnt, lead_ls[q]);
                add(rsl, rcnt, lead_rs[q]);
            }
            taken = lead;
            first = false;
        }
        int seen = 0;
        for (int64_t q = head; q < n && taken < 8 && seen < kWindow;) {
            const int64_t nq = nx[q];
            seen++;
            if (fits(lsl, lcnt, ls[q], lr[q]) && fits(rsl, rcnt, rs[q], rr[q])) {
                add(lsl, lcnt, ls[q]);
                add(rsl, rcnt, rs[q]);
                take(q);
                out.push_back(v[q]);
                taken++;
            }
            q = nq;
        }
        while (head < n && taken < 8) {
            const int64_t q = head;
            take(q);
            out.push_back(v[q]);
            taken++;
        }
    }
    v.swap(out);
}

// Scratch of the slab ordering, reused from tile to tile: a spring -> slab
// position table (open addressing; a slot is live when its stamp is the
// current round's) and the per-entry and per-set arrays of gather_permute.
struct PermuteScratch {
    std::vector<int64_t> hkey;
    std::vector<int32_t> hval;
    std::vector<uint32_t> hstamp;
    uint32_t stamp = 0;
    int64_t hcap = 0;
    std::vector<int64_t> seq;
    std::vector<int32_t> at, k0, k1;
    std::vector<uint8_t> cnt, mx;

    void begin(int64_t ne) {  // an empty table for up to ne springs
        int64_t c = 16;
        while (c < 2 * ne) c <<= 1;
        if ((int64_t)hkey.size() < c) {
            hkey.assign((size_t)c, -1);
            hval.assign((size_t)c, 0);
            hstamp.assign((size_t)c, 0);
            stamp = 0;
        }
        hcap = c;
        ++stamp;
    }
    size_t probe(int64_t sp) const {
        for (uint64_t h = ((uint64_t)sp * 0x9E3779B97F4A7C15ULL) >> 20;; h++) {
            const size_t q = (size_t)(h & (uint64_t)(hcap - 1));
            if (hstamp[q] != stamp || hkey[q] == sp) return q;
        }
    }
    void put(int64_t sp, int32_t v) {
        const size_t q = probe(sp);
        hkey[q] = sp;
        hval[q] = v;
        hstamp[q] = stamp;
    }
    int32_t get(int64_t sp) const { return hval[probe(sp)]; }
};

// Lowers the gather cost of a slab's within-group permutation by pairwise
// swaps.  A set (one quarter-warp's force loads at one incidence position)
// costs the most entries it reads from one bank group -- its wavefronts;
// two entries of one group (and one part) trade positions when that lowers
// the summed cost of their sets.  at: position -> entry; k0/k1: the entry's
// sets (-1: none); cnt: per set and residue, the entries read; mx:
// scratch for the sets' costs.  Sweeps over the groups repeat while one
// changes something, at most kSweeps times.
void swap_search(std::vector<int32_t> &at, const std::vector<int32_t> &k0, const std::vector<int32_t> &k1,
                 std::vector<uint8_t> &cnt, std::vector<uint8_t> &mx, int64_t na) {
    constexpr int kSweeps = 2;
    const int64_t ne = (int64_t)at.size(), nsets = (int64_t)(cnt.size() / 8);
    mx.resize((size_t)nsets);  // per set, its cost: the largest count
    for (int64_t st = 0; st < nsets; st++) mx[st] = *std::max_element(&cnt[st * 8], &cnt[st * 8] + 8);
    // change of a set's cost when one of its entries moves from residue
    // `from` to `to`: up when `to` is at the maximum, down when `from` is
    // the only residue at it and `to` stays below it
    auto delta = [&](int32_t st, int from, int to) {
        const uint8_t *c = &cnt[(size_t)st * 8];
        const int m = mx[st];
        if (c[to] == m) return 1;
        if (c[from] != m || c[to] + 1 == m) return 0;
        for (int r = 0; r < 8; r++)
            if (r != from && c[r] == m) return 0;
        return -1;
    };
    auto move = [&](int32_t st, int from, int to) {
        uint8_t *c = &cnt[(size_t)st * 8];
        c[from]--;
        c[to]++;
        mx[st] = *std::max_element(c, c + 8);
    };
    for (int sweep = 0; sweep < kSweeps; sweep++) {
        bool changed = false;
        for (int64_t b0 = 0; b0 < ne; b0 += 8) {
            const int64_t b1 = std::min<int64_t>(b0 + 8, ne);
            for (int side = 0; side < 2; side++) {
                const int64_t s0 = side == 0 ? b0 : std::max(b0, na), s1 = side == 0 ? std::min(b1, na) : b1;
                if (s1 - s0 < 2) continue;
                // a swap lowers the cost only if one of its entries is the
                // only one at the maximum (of 2 or more) of one of its sets
                bool drop[8];
                auto mark = [&]() {
                    for (int64_t p = s0; p < s1; p++) {
                        drop[p - s0] = false;
                        for (int32_t st : {k0[at[p]], k1[at[p]]}) {
                            if (st < 0) continue;
                            const uint8_t *c = &cnt[(size_t)st * 8];
                            if (mx[st] < 2 || c[p & 7] != mx[st]) continue;
                            int at_max = 0;
                            for (int r = 0; r < 8; r++) at_max += c[r] == mx[st];
                            drop[p - s0] = drop[p - s0] || at_max == 1;
                        }
                    }
                };
                mark();
                for (int64_t p = s0; p < s1; p++)
                    for (int64_t q = p + 1; q < s1; q++) {
                        if (!drop[p - s0] && !drop[q - s0]) continue;
                        const int32_t x = at[p], y = at[q];
                        const int rp = (int)(p & 7), rq = (int)(q & 7);
                        const int32_t sx[2] = {k0[x], k1[x]}, sy[2] = {k0[y], k1[y]};
                        auto in = [](const int32_t *v, int32_t st) { return v[0] == st || v[1] == st; };
                        int d = 0;  // a set holding both entries keeps its counts
                        for (int32_t st : sx)
                            if (st >= 0 && !in(sy, st)) d += delta(st, rp, rq);
                        for (int32_t st : sy)
                            if (st >= 0 && !in(sx, st)) d += delta(st, rq, rp);
                        if (d >= 0) continue;
                        for (int32_t st : sx)
                            if (st >= 0 && !in(sy, st)) move(st, rp, rq);
                        for (int32_t st : sy)
                            if (st >= 0 && !in(sx, st)) move(st, rq, rp);
                        std::swap(at[p], at[q]);
                        changed = true;
                        mark();
                    }
            }
        }
        if (!changed) break;
    }
}

// Permutes the entries inside each aligned group of eight slab positions
// (never across the actuated / non-actuated boundary), which keeps the
// grouping above, so that the force slots one quarter-warp gathers at one
// incidence position -- the j-th codes of eight consecutive masses, 16-byte
// loads of slots at bank group (slot mod 8) -- fall in distinct bank groups
// where they can.  Greedy per group first: the entries with the most gather
// references first, each to the free position whose residue the entry's
// (quarter-warp, j) sets use least; then swap_search.
void gather_permute(std::vector<int64_t> &act, std::vector<int64_t> &rest, int64_t lo, int64_t hi,
                    const std::vector<int64_t> &ip, const std::vector<int64_t> &isp, int64_t heavy_threshold,
                    PermuteScratch &W) {
    std::vector<int64_t> &seq = W.seq;
    seq.assign(act.begin(), act.end());
    seq.insert(seq.end(), rest.begin(), rest.end());
    const int64_t ne = (int64_t)seq.size(), na = (int64_t)act.size(), nm = hi - lo;
    if (ne <= 1) return;
    // spring -> position of this tile, in a small open-addressing table
    // (a global spring-indexed array would be read at scattered places)
    W.begin(ne);
    for (int64_t p = 0; p < ne; p++) W.put(seq[p], (int32_t)p);
    int64_t maxd = 1;
    for (int64_t m = lo; m < hi; m++) {
        const int64_t d = ip[m + 1] - ip[m];
        if (d <= heavy_threshold) maxd = std::max(maxd, d);
    }
    maxd = (maxd + 3) & ~int64_t(3);  // incidence positions, padding included
    // the (quarter-warp, incidence position) sets each entry belongs to
    std::vector<int32_t> &k0 = W.k0, &k1 = W.k1;
    k0.assign((size_t)ne, -1);
    k1.assign((size_t)ne, -1);
    for (int64_t m = lo; m < hi; m++) {
        const int64_t d = ip[m + 1] - ip[m];
        if (d > heavy_threshold) continue;
        for (int64_t j = 0; j < d; j++) {
            const int64_t p = W.get(isp[ip[m] + j]);
            const int32_t key = (int32_t)(((m - lo) >> 3) * maxd + j);
            if (k0[p] < 0) k0[p] = key;
            else if (k0[p] != key) k1[p] = key;  // both ends in one set: one broadcast load
        }
    }
    std::vector<uint8_t> &cnt = W.cnt;
    cnt.assign((size_t)(((nm + 7) >> 3) * maxd * 8), 0);
    // a mass's codes past its degree, up to a whole word of four, are
    // padding that the padded gathers load from slot ne: one fixed (and
    // broadcast) slot of those sets
    for (int64_t m = lo; m < hi; m++) {
        const int64_t d = ip[m + 1] - ip[m];
        if (d > heavy_threshold) continue;
        for (int64_t j = d; j < ((d + 3) & ~int64_t(3)); j++)
            cnt[(size_t)((((m - lo) >> 3) * maxd + j) * 8 + (ne & 7))] = 1;
    }
    std::vector<int32_t> &at = W.at;  // position -> entry (index into seq)
    at.assign((size_t)ne, 0);
    for (int64_t b0 = 0; b0 < ne; b0 += 8) {
        const int64_t b1 = std::min<int64_t>(b0 + 8, ne);
        for (int side = 0; side < 2; side++) {
            const int64_t s0 = side == 0 ? b0 : std::max(b0, na), s1 = side == 0 ? std::min(b1, na) : b1;
            if (s1 - s0 <= 0) continue;
            int64_t ord[8];  // the entries of positions s0..s1-1 (by their position in seq)
            int n8 = 0;
            for (int64_t x = s0; x < s1; x++) ord[n8++] = x;
            // most gather references first (stable insertion sort of <= 8)
            auto refs = [&](int64_t x) { return (k0[x] >= 0) + (k1[x] >= 0); };
            for (int q = 1; q < n8; q++)
                for (int r = q; r > 0 && refs(ord[r]) > refs(ord[r - 1]); r--) std::swap(ord[r], ord[r - 1]);
            bool taken[8] = {false};
            for (int q = 0; q < n8; q++) {
                const int64_t x = ord[q];
                // the entry's use of each residue, summed over its two sets
                // (eight byte counters added at once: each is at most 8)
                uint64_t c0 = 0, c1 = 0;
                if (k0[x] >= 0) std::memcpy(&c0, &cnt[(size_t)k0[x] * 8], 8);
                if (k1[x] >= 0) std::memcpy(&c1, &cnt[(size_t)k1[x] * 8], 8);
                const uint64_t cs = c0 + c1;
                int best = -1, bestc = 1 << 30;
                for (int64_t p = s0; p < s1; p++) {
                    if (taken[p - s0]) continue;
                    const int c = (int)((cs >> (8 * (p & 7))) & 0xff);
                    if (c < bestc) bestc = c, best = (int)(p - s0);
                }
                taken[best] = true;
                const int r = (int)((s0 + best) & 7);
                if (k0[x] >= 0) cnt[(size_t)k0[x] * 8 + r]++;
                if (k1[x] >= 0) cnt[(size_t)k1[x] * 8 + r]++;
                at[s0 + best] = (int32_t)x;
            }
        }
    }
    swap_search(at, k0, k1, cnt, W.mx, na);
    act.resize((size_t)na);
    rest.resize((size_t)(ne - na));
    for (int64_t p = 0; p < ne; p++) (p < na ? act[p] : rest[p - na]) = seq[at[p]];
}

// Runs f(state, i) for every i in [0, count) on up to planner_threads()
// host threads, each with its own State; at least `grain` items per thread.
// f may write only what belongs to item i.
// An exception in any thread stops the others taking items and is rethrown
// here once all have joined.
template <class State, class F>
void parallel_items(int64_t count, int64_t grain, F &&f) {
    const int nt = (int)std::min<int64_t>(planner_threads(), std::max<int64_t>(1, count / grain));
    std::atomic<int64_t> next{0};
    std::exception_ptr err;
    std::mutex err_mu;
    auto worker = [&]() {
        try {
            State state;
            for (int64_t i; (i = next.fetch_add(1)) < count;) f(state, i);
        } catch (...) {
            std::lock_guard<std::mutex> lk(err_mu);
            if (!err) err = std::current_exception();
            next.store(count);
        }
    };
    std::vector<std::thread> pool;
    for (int q = 1; q < nt; q++) {
        try {
            pool.emplace_back(worker);
        } catch (const std::system_error &) {
            break;  // no thread to be had: fewer threads take the items
        }
    }
    worker();
    for (auto &th : pool) th.join();
    if (err) std::rethrow_exception(err);
}

struct NoScratch {};

// One tile of the layout: masses [lo, hi); its slab entries (every spring
// that a free mass of the tile is an end of, once) in ascending spring
// order, actuated ones apart; the other ends outside the tile (its halo),
// ascending.
struct TileLayout {
    int64_t lo = 0, hi = 0;
    std::vector<int64_t> act, rest;
    std::vector<int32_t> halo;
};

// The tiles of one leaf: the leaf itself while its slab, halo and
// state records fit the tile limits, else its two halves (first half
// first, recursively).  err: a single mass whose slab does not fit.
struct LeafLayout {
    std::vector<TileLayout> tiles;
    std::string err;
};

struct LayoutScratch {
    std::vector<int64_t> ents;
    std::vector<int32_t> halo;
};

void layout_leaf(const PlanInput &in, const Plan &P, const std::vector<int32_t> &L, const std::vector<int32_t> &R,
                 const std::vector<int64_t> &ip, const std::vector<int64_t> &isp, int64_t lo0, int64_t hi0,
                 LeafLayout &out, LayoutScratch &S) {
    out.tiles.clear();
    out.err.clear();
    std::deque<std::pair<int64_t, int64_t>> work{{lo0, hi0}};
    while (!work.empty()) {
        const auto [lo, hi] = work.front();
        work.pop_front();
        const int64_t nm = hi - lo;
        // the incidence of masses lo..hi-1 is one range of isp
        S.ents.assign(isp.begin() + ip[lo], isp.begin() + ip[hi]);
        std::sort(S.ents.begin(), S.ents.end());
        S.ents.erase(std::unique(S.ents.begin(), S.ents.end()), S.ents.end());
        const int64_t ne = (int64_t)S.ents.size();
        bool fits = ne <= in.entry_cap;
        if (fits) {
            S.halo.clear();
            for (int64_t sp : S.ents)
                for (int32_t x : {L[sp], R[sp]})
                    if (x < lo || x >= hi) S.halo.push_back(x);
            std::sort(S.halo.begin(), S.halo.end());
            S.halo.erase(std::unique(S.halo.begin(), S.halo.end()), S.halo.end());
            fits = nm + (int64_t)S.halo.size() <= in.slot_cap;
            if (fits) {
                int64_t heavy = 0;
                for (int64_t m = lo; m < hi; m++) heavy += (ip[m + 1] - ip[m]) > in.heavy_threshold;
                fits = (nm + (int64_t)S.halo.size()) * in.slot_bytes + (ne + 1) * in.entry_bytes +
                           heavy * in.heavy_bytes <= in.smem_budget;
            }
        }
        if (!fits) {
            if (nm == 1) {
                out.err = "mass " + std::to_string(P.new2old[lo]) + " has " + std::to_string(ip[lo + 1] - ip[lo]) +
                          " springs, more than one tile's slab can hold";
                return;
            }
            const int64_t mid = lo + nm / 2;
            work.emplace_front(mid, hi);
            work.emplace_front(lo, mid);
            continue;
        }
        TileLayout t;
        t.lo = lo;
        t.hi = hi;
        for (int64_t sp : S.ents) (actuated(in, sp) ? t.act : t.rest).push_back(sp);
        t.halo = S.halo;
        out.tiles.push_back(std::move(t));
    }
}

// Final slab order of tile t (bank_order on each part, then
// gather_permute), its entry words, and the incidence codes of its masses
// (ELL block and heavy lists), written into the tile's own ranges of P's
// tables, which the sequential pass laid out (entries in spring order, code
// slots, heavy lists).
void order_tile(const PlanInput &in, Plan &P, int64_t t, const std::vector<int32_t> &L,
                const std::vector<int32_t> &R, const std::vector<int64_t> &ip, const std::vector<int64_t> &isp,
                const std::vector<int8_t> &isg, PermuteScratch &W) {
    const int64_t lo = P.tile_mass_off[t], hi = P.tile_mass_off[t + 1], nm = hi - lo;
    const int64_t e0 = P.tile_ent_off[t], e1 = P.tile_ent_off[t + 1], na = P.tile_nact[t];
    const int32_t *halo = P.halo.data() + P.tile_halo_off[t];
    const int64_t nh = P.tile_nh[t];
    auto slot = [&](int32_t x) -> uint32_t {  // tile masses, then the sorted halo
        if (x >= lo && x < hi) return (uint32_t)(x - lo);
        return (uint32_t)(nm + (std::lower_bound(halo, halo + nh, x) - halo));
    };
    std::vector<int64_t> ents_act(P.ent_spring.begin() + e0, P.ent_spring.begin() + e0 + na);
    std::vector<int64_t> ents(P.ent_spring.begin() + e0 + na, P.ent_spring.begin() + e1);
    {
        // the non-actuated part continues the actuated part's last group
        uint32_t lead_ls[8], lead_rs[8];
        int lead = 0;
        for (auto *v : {&ents_act, &ents}) {
            std::vector<uint32_t> ls(v->size()), rs(v->size());
            for (size_t q = 0; q < v->size(); q++) {
                ls[q] = slot(L[(*v)[q]]);
                rs[q] = slot(R[(*v)[q]]);
            }
            bank_order(*v, ls, rs, in.slot_bytes, lead_ls, lead_rs, lead);
            // the open group after this part: its last (lead + size) % 8
            // entries of the carried ones followed by this part's
            std::vector<uint32_t> cl(lead_ls, lead_ls + lead), cr(lead_rs, lead_rs + lead);
            for (int64_t sp : *v) {
                cl.push_back(slot(L[sp]));
                cr.push_back(slot(R[sp]));
            }
            const int tail = (int)(cl.size() % 8);
            std::copy(cl.end() - tail, cl.end(), lead_ls);
            std::copy(cr.end() - tail, cr.end(), lead_rs);
            lead = tail;
        }
    }
    gather_permute(ents_act, ents, lo, hi, ip, isp, in.heavy_threshold, W);
    W.begin(e1 - e0);
    int64_t e = e0;
    for (auto *v : {&ents_act, &ents})
        for (int64_t sp : *v) {
            W.put(sp, (int32_t)(e - e0));
            P.ent_spring[e] = sp;
            P.ent_ends[e] = pack_ends(slot(L[sp]), slot(R[sp]), in.type ? (uint32_t)in.type[sp] : 0u);
            e++;
        }
    auto code_of = [&](int64_t q) -> uint16_t { return (uint16_t)(W.get(isp[q]) | (isg[q] < 0 ? 0x8000 : 0)); };
    int64_t hv = P.tile_heavy_off[t];
    for (int64_t w = P.tile_warp_off[t]; w < P.tile_warp_off[t + 1]; w++) {
        const int64_t m0 = lo + 32 * (w - P.tile_warp_off[t]), m1 = std::min(m0 + 32, hi);
        const uint32_t off = P.warp_inc_off[w];
        for (int64_t m = m0; m < m1; m++) {
            const int64_t d = ip[m + 1] - ip[m];
            if (d <= in.heavy_threshold) {
                for (int64_t j = 0; j < d; j++)
                    P.inc[ell_index(off, (uint32_t)(m - m0), (uint32_t)j)] = code_of(ip[m] + j);
            } else {
                const uint32_t h0 = P.heavy_inc_off[hv++];
                for (int64_t q = ip[m]; q < ip[m + 1]; q++) P.heavy_inc[h0 + (q - ip[m])] = code_of(q);
            }
        }
    }
}


}  // namespace

static std::string build_plan_tables(const PlanInput &in, Plan &P) {
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

    // ---- spatial order inside each body ----------------------------------
    // Each body is cut by recursive coordinate bisection of its start pose
    // into ceil(size / tile) near-cubic leaves (the longest side of a
    // leaf's box is split so that each side gets its share of whole tiles),
    // and the masses of a leaf are put in Morton order.  A leaf is a tile
    // unless the shared-memory budget splits it further: near-cubic tiles
    // have less halo and fewer cross-tile springs than runs of a Morton
    // curve (100^3 lattice, tile 192: 17 % smaller halos, 4 % fewer slab
    // entries).  Coordinates are quantised to 21 bits per axis (non-finite
    // ones to 0), which also makes the cut independent of rounding.
    P.new2old.resize(n);
    std::iota(P.new2old.begin(), P.new2old.end(), 0);
    std::vector<uint64_t> code(n, 0);
    std::vector<uint32_t> qc(3 * (size_t)n, 0);
    std::vector<int64_t> leaf_end;  // new-index end of each leaf, in order
    // bodies on several threads (each writes only its own ranges); a lone
    // body cuts its top levels on several threads instead
    std::vector<std::vector<int64_t>> body_leaves((size_t)P.nbodies);
    parallel_items<NoScratch>(P.nbodies, 16, [&](NoScratch &, int64_t b) {
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
                qc[3 * i + c] = (uint32_t)q[c];
            }
            code[i] = spread21(q[0]) | (spread21(q[1]) << 1) | (spread21(q[2]) << 2);
        }
        const int cap_b = (b1 - b0) <= (int64_t)in.whole_cap ? (int)(b1 - b0) : in.tile_cap;
        int depth = 0;  // a lone body: about one cut's half per thread
        while (P.nbodies == 1 && (2 << depth) <= planner_threads() && depth < 6) depth++;
        bisect(P.new2old.data() + b0, b1 - b0, cap_b, qc, code, b0, body_leaves[b], depth);
    });
    for (const auto &v : body_leaves) leaf_end.insert(leaf_end.end(), v.begin(), v.end());
    P.old2new.resize(n);
    for (int64_t i = 0; i < n; i++) P.old2new[P.new2old[i]] = (int32_t)i;

    // ---- springs in the new numbering -----------------------------------
    // (chunks of springs on several threads)
    constexpr int64_t kChunk = 1 << 16;
    const int64_t nchunks = (ns + kChunk - 1) / kChunk;
    std::vector<int32_t> L(ns, -1), R(ns, -1);
    std::vector<int64_t> chunk_valid((size_t)nchunks, 0);
    parallel_items<NoScratch>(nchunks, 4, [&](NoScratch &, int64_t c) {
        for (int64_t s = c * kChunk; s < std::min(ns, (c + 1) * kChunk); s++) {
            int32_t l = in.left[s], r = in.right[s];
            if (l < 0 || r < 0 || l >= n || r >= n) continue;  // skipped as src/sim.cu:1052 does
            L[s] = P.old2new[l];
            R[s] = P.old2new[r];
            chunk_valid[c]++;
        }
    });
    for (int64_t v : chunk_valid) P.valid_springs += v;
    std::vector<uint8_t> fixed_new(n, 0);
    if (in.fixed)
        for (int64_t m = 0; m < n; m++) fixed_new[m] = in.fixed[P.new2old[m]] ? 1 : 0;

    // incidence of each (non-fixed) mass, ascending spring order; for a spring
    // attached twice to one mass the right end comes first (src/sim.cu:1067-1077).
    // Counted and filled on several threads, then each mass's list sorted.
    std::vector<std::atomic<int64_t>> fillc((size_t)n);  // value-initialised: zero
    parallel_items<NoScratch>(nchunks, 4, [&](NoScratch &, int64_t c) {
        for (int64_t s = c * kChunk; s < std::min(ns, (c + 1) * kChunk); s++) {
            if (L[s] < 0) continue;
            if (!fixed_new[R[s]]) fillc[R[s]].fetch_add(1, std::memory_order_relaxed);
            if (!fixed_new[L[s]]) fillc[L[s]].fetch_add(1, std::memory_order_relaxed);
        }
    });
    std::vector<int64_t> ip(n + 1, 0);
    for (int64_t i = 0; i < n; i++) {
        ip[i + 1] = ip[i] + fillc[i].load(std::memory_order_relaxed);
        fillc[i].store(ip[i], std::memory_order_relaxed);
    }
    std::vector<int64_t> isp(ip[n]);
    std::vector<int8_t> isg(ip[n]);
    parallel_items<NoScratch>(nchunks, 4, [&](NoScratch &, int64_t c) {
        for (int64_t s = c * kChunk; s < std::min(ns, (c + 1) * kChunk); s++) {
            if (L[s] < 0) continue;
            if (!fixed_new[R[s]]) {
                const int64_t q = fillc[R[s]].fetch_add(1, std::memory_order_relaxed);
                isp[q] = s;
                isg[q] = 1;
            }
            if (!fixed_new[L[s]]) {
                const int64_t q = fillc[L[s]].fetch_add(1, std::memory_order_relaxed);
                isp[q] = s;
                isg[q] = -1;
            }
        }
    });
    {
        constexpr int64_t kMassChunk = 1 << 14;
        parallel_items<NoScratch>((n + kMassChunk - 1) / kMassChunk, 4, [&](NoScratch &, int64_t c) {
            std::vector<std::pair<int64_t, int8_t>> v;
            for (int64_t m = c * kMassChunk; m < std::min(n, (c + 1) * kMassChunk); m++) {
                v.clear();
                for (int64_t q = ip[m]; q < ip[m + 1]; q++) v.emplace_back(isp[q], isg[q]);
                // ascending spring; right end (+1) before left end (-1)
                std::sort(v.begin(), v.end(), [](const auto &a, const auto &b) {
                    return a.first < b.first || (a.first == b.first && a.second > b.second);
                });
                for (int64_t q = ip[m]; q < ip[m + 1]; q++) {
                    isp[q] = v[q - ip[m]].first;
                    isg[q] = v[q - ip[m]].second;
                }
            }
        });
    }

    // ---- tiles ------------------------------------------------------------
    // Leaves are laid out on several threads, a batch at a time (bounded
    // memory), and their tiles appended to the tables in leaf order.
    P.tile_mass_off.push_back(0);
    P.tile_halo_off.push_back(0);
    P.tile_ent_off.push_back(0);
    P.tile_warp_off.push_back(0);
    P.tile_heavy_off.push_back(0);
    P.deg.assign(n, 0);

    const int64_t nleaves = (int64_t)leaf_end.size();
    std::vector<int32_t> leaf_body((size_t)nleaves);
    for (int64_t f = 0, b = 0; f < nleaves; f++) {
        while (leaf_end[f] > bptr[b + 1]) b++;
        leaf_body[f] = (int32_t)b;
    }
    // capacity: the tiles' entries are at most all incidences; the incidence
    // blocks are about as many codes plus the padding of each warp's width
    P.ent_spring.reserve((size_t)ip[n]);
    P.ent_ends.reserve((size_t)ip[n]);
    P.inc.reserve((size_t)(ip[n] + 4 * n));
    constexpr int64_t kLeafBatch = 4096;
    std::vector<LeafLayout> batch;
    for (int64_t f0 = 0; f0 < nleaves; f0 += kLeafBatch) {
        const int64_t nb = std::min(kLeafBatch, nleaves - f0);
        batch.resize((size_t)nb);
        parallel_items<LayoutScratch>(nb, 8, [&](LayoutScratch &S, int64_t i) {
            const int64_t f = f0 + i;
            layout_leaf(in, P, L, R, ip, isp, f == 0 ? 0 : leaf_end[f - 1], leaf_end[f], batch[i], S);
        });
        for (int64_t i = 0; i < nb; i++) {
            if (!batch[i].err.empty()) return batch[i].err;
            for (const TileLayout &T : batch[i].tiles) {
                // the tile's slab order, entry words and incidence codes are
                // filled in by order_tile() below
                const int64_t lo = T.lo, hi = T.hi, nm = hi - lo;
                const int64_t nh = (int64_t)T.halo.size();
                const int64_t ne = (int64_t)(T.act.size() + T.rest.size());
                for (auto *v : {&T.act, &T.rest}) P.ent_spring.insert(P.ent_spring.end(), v->begin(), v->end());
                P.ent_ends.resize(P.ent_spring.size(), 0u);
                P.halo.insert(P.halo.end(), T.halo.begin(), T.halo.end());
                while (P.halo.size() % 4) P.halo.push_back(T.halo.empty() ? (int32_t)lo : T.halo.back());
                P.tile_nh.push_back((int32_t)nh);
                P.tile_nact.push_back((int32_t)T.act.size());

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
                    P.warp_inc_off.push_back((uint32_t)P.inc.size());
                    // padding codes name slot ne, one past the tile's entries: a
                    // kernel that keeps a zero force there can sum whole words
                    P.inc.resize(P.inc.size() + (size_t)(width * 32), (uint16_t)ne);
                    for (int64_t m = m0; m < m1; m++) {
                        int64_t d = ip[m + 1] - ip[m];
                        if (d <= in.heavy_threshold) {
                            P.deg[m] = (uint8_t)d;
                        } else {
                            P.deg[m] = 255;
                            P.heavy_local.push_back((uint16_t)(m - lo));
                            P.heavy_inc_off.push_back((uint32_t)P.heavy_inc.size());
                            P.heavy_inc.resize(P.heavy_inc.size() + (size_t)d, 0);
                            nheavy++;
                        }
                    }
                }
                P.body_of_tile.push_back(leaf_body[f0 + i]);
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
    }
    P.heavy_inc_off.push_back((uint32_t)P.heavy_inc.size());
    P.ntiles = (int64_t)P.body_of_tile.size();

    // ---- slab order, entry words and incidence codes, tiles in parallel ---
    // (each tile writes only its own ranges of the tables)
    parallel_items<PermuteScratch>(P.ntiles, 8, [&](PermuteScratch &W, int64_t t) {
        order_tile(in, P, t, L, R, ip, isp, isg, W);
    });
    return "";
}

std::string build_plan(const PlanInput &in, Plan &P) {
    try {
        return build_plan_tables(in, P);
    } catch (const std::bad_alloc &) {
        P = Plan();
        return "host memory exhausted while planning";
    } catch (const std::exception &e) {
        P = Plan();
        return std::string("planning failed: ") + e.what();
    }
}

void build_resident(const PlanInput &in, const Plan &P, int max_masses, int bin_cap, ResPlan &R) {
    R = ResPlan();
    const int64_t n = P.n;
    std::vector<int64_t> bptr;
    if (in.nbodies > 0 && in.body_ptr)
        bptr.assign(in.body_ptr, in.body_ptr + in.nbodies + 1);
    else
        bptr = {0, n};
    const int64_t nb = (int64_t)bptr.size() - 1;
    R.resident.assign(nb, 0);
    R.tile_resident.assign(P.ntiles, 0);
    max_masses = std::min(max_masses, 32767);
    bin_cap = std::max(std::min(bin_cap, 32767), 1);
    max_masses = std::min(max_masses, bin_cap);
    R.bin_cap = bin_cap;
    auto fixed_new = [&](int64_t g) { return in.fixed && in.fixed[P.new2old[g]]; };
    // bodies occupy contiguous ranges of the tiled order (tiles never
    // straddle bodies and masses are only reordered inside a body)
    std::vector<int32_t> body_of(n);
    for (int64_t b = 0; b < nb; b++)
        for (int64_t g = bptr[b]; g < bptr[b + 1]; g++) body_of[g] = (int32_t)b;
    // incidence of each free mass in the new numbering, ascending springs
    std::vector<int64_t> ip(n + 1, 0);
    std::vector<uint8_t> cross(nb, 0);
    for (int64_t s = 0; s < in.ns; s++) {
        int32_t l = in.left[s], r = in.right[s];
        if (l < 0 || r < 0 || l >= n || r >= n) continue;
        int64_t L = P.old2new[l], Rr = P.old2new[r];
        if (body_of[L] != body_of[Rr]) cross[body_of[L]] = cross[body_of[Rr]] = 1;
        if (!fixed_new(Rr)) ip[Rr + 1]++;
        if (!fixed_new(L)) ip[L + 1]++;
    }
    for (int64_t i = 0; i < n; i++) ip[i + 1] += ip[i];
    std::vector<int64_t> isp(ip[n]), iother(ip[n]);
    std::vector<int8_t> iright(ip[n]);
    {
        std::vector<int64_t> fill(ip.begin(), ip.end() - 1);
        for (int64_t s = 0; s < in.ns; s++) {
            int32_t l = in.left[s], r = in.right[s];
            if (l < 0 || r < 0 || l >= n || r >= n) continue;
            int64_t L = P.old2new[l], Rr = P.old2new[r];
            if (!fixed_new(Rr)) { isp[fill[Rr]] = s; iother[fill[Rr]] = L; iright[fill[Rr]] = 1; fill[Rr]++; }
            if (!fixed_new(L)) { isp[fill[L]] = s; iother[fill[L]] = Rr; iright[fill[L]] = 0; fill[L]++; }
        }
    }
    // eligible bodies, largest first (ties: body order)
    std::vector<int64_t> elig;
    for (int64_t b = 0; b < nb; b++) {
        const int64_t nm = bptr[b + 1] - bptr[b];
        if (nm > max_masses || cross[b]) continue;
        bool ok = true;
        for (int64_t g = bptr[b]; g < bptr[b + 1] && ok; g++) ok = ip[g + 1] - ip[g] <= 254;
        if (ok) elig.push_back(b);
    }
    std::stable_sort(elig.begin(), elig.end(),
                     [&](int64_t a, int64_t b) { return bptr[a + 1] - bptr[a] > bptr[b + 1] - bptr[b]; });
    // best fit: the fullest bin the body still fits in
    std::multimap<int64_t, int64_t> room;  // remaining capacity -> bin
    std::vector<std::vector<int64_t>> bins;
    for (int64_t b : elig) {
        const int64_t nm = bptr[b + 1] - bptr[b];
        auto it = room.lower_bound(nm);
        int64_t k;
        if (it == room.end()) {
            k = (int64_t)bins.size();
            bins.emplace_back();
        } else {
            k = it->second;
            room.erase(it);
        }
        bins[k].push_back(b);
        int64_t used = 0;
        for (int64_t q : bins[k]) used += bptr[q + 1] - bptr[q];
        if (bin_cap - used > 0) room.emplace(bin_cap - used, k);
        R.resident[b] = 1;
    }
    // bins with the most incidence work first
    std::vector<int64_t> work(bins.size(), 0), order(bins.size());
    for (size_t k = 0; k < bins.size(); k++)
        for (int64_t b : bins[k]) work[k] += ip[bptr[b + 1]] - ip[bptr[b]] + (bptr[b + 1] - bptr[b]);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return work[a] > work[b]; });
    R.nbins = (int64_t)bins.size();
    R.bin_mass_off.push_back(0);
    R.bin_warp_off.push_back(0);
    std::vector<int64_t> local(n, -1);
    for (int64_t k : order) {
        const int64_t m0 = (int64_t)R.mass.size();
        for (int64_t b : bins[k]) {
            R.nbodies++;
            for (int64_t g = bptr[b]; g < bptr[b + 1]; g++) {
                local[g] = (int64_t)R.mass.size() - m0;
                R.mass.push_back((int32_t)g);
                R.body.push_back((int32_t)b);
            }
        }
        const int64_t m1 = (int64_t)R.mass.size();
        for (int64_t w0 = m0; w0 < m1; w0 += 32) {
            const int64_t w1 = std::min(w0 + 32, m1);
            int64_t width = 0;
            for (int64_t q = w0; q < w1; q++) {
                const int64_t g = R.mass[q];
                width = std::max(width, ip[g + 1] - ip[g]);
            }
            const uint32_t off = (uint32_t)R.words.size();
            R.warp_rec_off.push_back(off);
            R.words.resize(R.words.size() + (size_t)(width * 32), 0);
            R.rec_spring.resize(R.words.size(), -1);
            for (int64_t q = w0; q < w1; q++) {
                const int64_t g = R.mass[q], lane = q - w0, d = ip[g + 1] - ip[g];
                uint64_t mask = 0;
                for (int64_t j = 0; j < d; j++) {
                    const int64_t e = ip[g] + j, s = isp[e];
                    const uint32_t other = (uint32_t)local[iother[e]];
                    const uint32_t ty = in.type ? (uint32_t)in.type[s] & 3u : 0u;
                    R.words[off + j * 32 + lane] = other | (iright[e] ? 0x8000u : 0u) | (ty << 16);
                    R.rec_spring[off + j * 32 + lane] = s;
                    if (j < 64 && ty >= 2) mask |= uint64_t(1) << j;
                }
                R.deg.push_back((uint8_t)d);
                R.act_mask.push_back(mask);
            }
        }
        R.bin_mass_off.push_back(m1);
        R.bin_warp_off.push_back((int64_t)R.warp_rec_off.size());
    }
    R.nmasses = (int64_t)R.mass.size();
    for (int64_t t = 0; t < P.ntiles; t++) R.tile_resident[t] = R.resident[P.body_of_tile[t]];
}

std::string build_pull(const Plan &P, const std::vector<PullTile> &tiles, int team_warps, int rec_f4,
                       const PullSprings &sp, PullTables &T) try {
    T = PullTables();
    T.team_warps = team_warps;
    const int64_t nt = (int64_t)tiles.size();
    const int64_t nu = nt * team_warps;
    auto code_of = [&](const PullTile &ti, int64_t u, int l, int j) {
        return P.inc[ell_index(P.warp_inc_off[ti.warp_off + u], (uint32_t)l, (uint32_t)j)];
    };
    // pass 1: per unit slot its masses, columns and whether damping varies
    std::vector<uint16_t> nq(nu, 0);
    std::vector<uint8_t> lanes(nu, 0), damp(nu, 0), heavy(nu, 0);
    std::vector<float> damp0(nu, 0.f);
    parallel_items<NoScratch>(nu, 256, [&](NoScratch &, int64_t q) {
        const PullTile &ti = tiles[q / team_warps];
        const int64_t u = q % team_warps;
        if (32 * u >= ti.nm) return;
        lanes[q] = (uint8_t)std::min<int64_t>(32, ti.nm - 32 * u);
        int nc = 0;
        bool first = true;
        for (int l = 0; l < lanes[q]; l++) {
            const int d = P.deg[ti.mass_off + 32 * u + l];
            if (d == 255) {
                heavy[q] = 1;
                return;
            }
            nc = std::max(nc, d);
            for (int j = 0; j < d; j++) {
                const int64_t sj = P.ent_spring[ti.ent_off + (code_of(ti, u, l, j) & 0x7fff)];
                const float c = sp.damping ? (float)sp.damping[sj] : 0.f;
                if (first) {
                    damp0[q] = c;
                    first = false;
                } else if (std::memcmp(&c, &damp0[q], 4) != 0) {
                    damp[q] = 1;
                }
            }
        }
        nq[q] = (uint16_t)((nc + 3) / 4);
    });
    for (int64_t q = 0; q < nu; q++)
        if (heavy[q]) return "a mass of degree above the heavy threshold (the pull form has no warp-cooperative sums)";
    std::vector<uint64_t> off(nu + 1, 0);
    for (int64_t q = 0; q < nu; q++) off[q + 1] = off[q] + (uint64_t)nq[q] * pull_quad_bytes(damp[q] != 0);
    if (off[nu] / 128 > UINT32_MAX) return "pull tables exceed their 32-bit offsets";
    T.units.assign(nu, PullUnit{});
    T.ell.assign(std::max<uint64_t>(off[nu], 128), 0);
    // pass 2: fill
    parallel_items<NoScratch>(nu, 256, [&](NoScratch &, int64_t q) {
        const PullTile &ti = tiles[q / team_warps];
        const int64_t u = q % team_warps;
        PullUnit &pu = T.units[q];
        pu.ell = (uint32_t)(off[q] / 128);
        pu.nquads = nq[q];
        pu.lanes = lanes[q];
        pu.flags = damp[q] ? PU_DAMP : 0;
        pu.damping = damp[q] ? 0.f : damp0[q];
        pu.mass0 = (int32_t)(ti.mass_off + 32 * u);
        const uint32_t qb = pull_quad_bytes(damp[q] != 0);
        for (int l = 0; l < lanes[q]; l++) {
            const int d = P.deg[ti.mass_off + 32 * u + l];
            for (int j = 0; j < d; j++) {
                uint8_t *blk = T.ell.data() + off[q] + (uint64_t)(j / 4) * qb;
                const int c = j % 4;
                const uint16_t code = code_of(ti, u, l, j);
                const uint32_t e_local = code & 0x7fffu;
                const uint32_t ends = P.ent_ends[ti.ent_off + e_local];
                const uint32_t ls = ends & 0xfffu, rs = (ends >> 12) & 0xfffu, ty = (ends >> 24) & 3u;
                const uint32_t nbr = (code & 0x8000) ? rs : ls;
                const int64_t sj = P.ent_spring[ti.ent_off + e_local];
                const bool act = ty >= 2;
                const uint16_t w = (uint16_t)((nbr * (uint32_t)rec_f4) | PW_VALID | (act ? PW_ACT : 0u));
                std::memcpy(blk + 8 * l + 2 * c, &w, 2);
                const float kf = (float)sp.k[sj];
                std::memcpy(blk + 256 + 16 * l + 4 * c, &kf, 4);
                if (act) {
                    std::memcpy(blk + 768 + 16 * l + 4 * c, &e_local, 4);
                } else {
                    const float rf = (float)sp.rest[sj];
                    std::memcpy(blk + 768 + 16 * l + 4 * c, &rf, 4);
                }
                if (damp[q]) {
                    const float cf = sp.damping ? (float)sp.damping[sj] : 0.f;
                    std::memcpy(blk + 1280 + 16 * l + 4 * c, &cf, 4);
                }
            }
        }
    });
    return "";
} catch (const std::bad_alloc &) {
    return "host memory exhausted";
}

}  // namespace tg
