// Runs the matcher's device core (graphpi_gb300/csrc/match_core.cuh) on
// emulated warps (warp_emu.h) over small skewed graphs and compares every
// per-pattern count with the CPU oracle (oracle/oracle.c).  Built with
// AddressSanitizer by tests/test_emu.py.  Every per-warp scratch region and
// every set slot is followed by a poisoned guard, so a set written past its
// slot or a warp past its region is reported at the faulting access.
//
//   emu_match [case ...]     cases: quick, donation, leafslices, pair,
//                            pairhub, pairtags, stripes, vec, rows
//                            (default: all but donation and leafslices)
#include <sanitizer/asan_interface.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gpm_gen.h"
#include "gpm_internal.h"
// last: its CUDA keyword macros must not reach the system headers
#include "warp_emu.h"

namespace gpm {
#include "match_core.cuh"
#include "csr_rows.cuh"
}

extern "C" int oracle_pattern_matching(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw,
                                       int threads, uint64_t* out);
extern "C" long long oracle_triangle_count(int V, const uint32_t* rp, const int32_t* col, int threads);

using namespace gpm;

namespace {

#ifndef ASAN_POISON_MEMORY_REGION
#define ASAN_POISON_MEMORY_REGION(a, s) ((void)(a), (void)(s))
#define ASAN_UNPOISON_MEMORY_REGION(a, s) ((void)(a), (void)(s))
#endif

constexpr int kGuard = 16;  // poisoned ints after every slot and warp region
int failures = 0;

struct Csr {
    int v = 0;
    std::vector<uint32_t> rp;
    std::vector<int32_t> col;
    int max_deg = 0;
};

Csr take(uint32_t* rp, int32_t* col, int v) {
    Csr g;
    g.v = v;
    g.rp.assign(rp, rp + v + 1);
    g.col.assign(col, col + rp[v]);
    for (int i = 0; i < v; ++i) g.max_deg = std::max<int>(g.max_deg, (int)(rp[i + 1] - rp[i]));
    gpm_free(rp);
    gpm_free(col);
    return g;
}

Csr relabelled(const Csr& in) {
    uint32_t* rp = nullptr;
    int32_t* col = nullptr;
    if (gpm_csr_relabel_degree(in.v, in.rp.data(), in.col.data(), &rp, &col)) std::abort();
    return take(rp, col, in.v);
}

Csr rmat(int scale, int ef, uint64_t seed) {
    uint32_t* rp = nullptr;
    int32_t* col = nullptr;
    int v = 0;
    if (gpm_gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed, &rp, &col, &v)) std::abort();
    return relabelled(take(rp, col, v));
}

Csr chung_lu(int n, double avg, double gamma, int maxd, uint64_t seed) {
    uint32_t* rp = nullptr;
    int32_t* col = nullptr;
    int v = 0;
    if (gpm_gen_chung_lu(n, avg, gamma, maxd, seed, &rp, &col, &v)) std::abort();
    return relabelled(take(rp, col, v));
}

struct Sched {
    std::vector<int64_t> tables;
    DevPlan plan;
};

std::vector<Sched> motif_schedules(const Csr& g, int k, bool iep, int stride) {
    std::vector<int32_t> adj(1 << 16);
    int count = 0;
    if (gpm_motifs(k, adj.data(), (int)adj.size(), &count)) std::abort();
    const long long tri = oracle_triangle_count(g.v, g.rp.data(), g.col.data(), 0);
    std::vector<Sched> out;
    for (int m = 0; m < count; m += stride) {
        Sched s;
        s.tables.resize(4096);
        int nw = 0, valid = 0;
        if (gpm_schedule_build(k, adj.data() + (size_t)m * k * k, 1, 1, iep ? 1 : 0, g.v, g.rp[g.v], tri,
                               s.tables.data(), (int)s.tables.size(), &nw, &valid))
            std::abort();
        if (!valid) continue;
        s.tables.resize(nw);
        if (compile_plan(s.tables.data(), nw, &s.plan)) std::abort();
        out.push_back(s);
    }
    return out;
}

struct Knobs {
    int blocks = 2, wpb = 4, chunk = 2, stage_cap = 64, leaf = 1, pair = 0, split = 0, pair_log2 = 13;
    int bm_min = 0;  // > 0: leaf bitmaps for fixed sets of at least this size
    int dense = 0;   // > 0: that many dense counter arrays for big pair sums
    unsigned long long stripes = 1, stripe = 0;
    // pair-sum tables kept across launches (their stored tags too), as the
    // engine keeps them; null: fresh zeroed tables for this launch
    std::vector<unsigned long long>* keep_tables = nullptr;
};

// One emulated launch over all pairs; returns the raw 128-bit sums.
std::vector<__int128> launch(const Csr& g, const std::vector<Sched>& ss, const Knobs& k) {
    const int n = (int)ss.size();
    int nslots = 1;
    for (const Sched& s : ss) nslots = std::max(nslots, s.plan.nslots);
    const int cap = std::max(1, g.max_deg) + kGuard;  // slot stride; the last kGuard ints are poisoned
    // slots, a poisoned guard, then the pair sums' block-sum tail (the
    // kernel finds the tail at the end of each warp's region)
    const long long per_warp = (long long)nslots * cap + kGuard + 2 * pair_bs_stride(cap);
    const int warps = k.blocks * k.wpb;
    std::vector<int> scratch((size_t)warps * per_warp);
    for (int w = 0; w < warps; ++w) {
        int* base = scratch.data() + (size_t)w * per_warp;
        for (int s = 0; s < nslots; ++s) ASAN_POISON_MEMORY_REGION(base + (size_t)s * cap + (cap - kGuard), kGuard * 4);
        ASAN_POISON_MEMORY_REGION(base + (size_t)nslots * cap, kGuard * 4);
    }
    std::vector<PairDesc> pairs(n);
    for (int i = 0; i < n; ++i) {
        pairs[i].g.rowptr = g.rp.data();
        pairs[i].g.col = g.col.data();
        pairs[i].g.v_cnt = g.v;
        pairs[i].g.pad_ = 0;
        pairs[i].g.e_cnt = g.rp[g.v];
        pairs[i].plan = &ss[i].plan;
        pairs[i].ntasks = ss[i].plan.T == 1 ? (unsigned long long)g.v : (unsigned long long)g.rp[g.v];
        pairs[i].cap = cap;
        pairs[i].pad_ = 0;
    }
    std::vector<unsigned long long> cursors(n, 0), out(2 * n, 0), stats(2, 0);
    unsigned long long params[2] = {k.stripes, k.stripe};
    std::vector<unsigned long long> tables;
    // the tables, then one stored tag per warp (zero: fresh tables)
    const size_t table_words = ((size_t)warps << k.pair_log2) + (size_t)warps;
    if (k.pair && k.keep_tables && k.keep_tables->size() != table_words) k.keep_tables->assign(table_words, 0ull);
    if (k.pair && !k.keep_tables) tables.assign(table_words, 0ull);
    unsigned long long* tab = !k.pair ? nullptr : (k.keep_tables ? k.keep_tables->data() : tables.data());
    const int bm_words = k.bm_min > 0 ? (g.v + 31) / 32 : 0;
    // dense pool: lock words padded to 64, then k.dense arrays of g.v counters
    std::vector<unsigned> dense(k.dense ? 64 + (size_t)k.dense * g.v : 0, 0u);
    std::vector<unsigned> bitmaps((size_t)warps * 2 * bm_words, 0u);
    DonationArea* don = k.split > 0 ? new DonationArea() : nullptr;
    if (don) std::memset((void*)don, 0, sizeof(DonationArea));
    const size_t smem = sizeof(WarpState) * k.wpb + sizeof(int) * 2 * (size_t)stage_stride(k.stage_cap) * k.wpb;
    std::vector<std::vector<unsigned char>> shared(k.blocks, std::vector<unsigned char>(smem));
    gpm_emu::block_dim = {(unsigned)(k.wpb * 32), 1, 1};
    gpm_emu::grid_dim = {(unsigned)k.blocks, 1, 1};
    std::atomic<int> done{0};
    std::vector<std::thread> th;
    for (int b = 0; b < k.blocks; ++b)
        for (int wi = 0; wi < k.wpb; ++wi)
            th.emplace_back([&, b, wi] {
                gpm_emu::Warp* w = new gpm_emu::Warp();
                for (int l = 0; l < 32; ++l) {
                    w->th[l].tid = {(unsigned)(wi * 32 + l), 0, 0};
                    w->th[l].bid = {(unsigned)b, 0, 0};
                    w->th[l].smem = shared[b].data();
                }
                auto body = [&](int) {
                    match_kernel<false, 1>(pairs.data(), n, cursors.data(), out.data(), scratch.data(), per_warp, k.chunk,
                                        params, k.leaf, k.stage_cap, k.pair, tab, k.pair_log2, don,
                                        k.split, bm_words ? bitmaps.data() : nullptr, bm_words, k.bm_min,
                                        k.dense ? dense.data() : nullptr, k.dense, g.v, stats.data());
                };
                gpm_emu::run_warp(*w, body);
                delete w;
                done.fetch_add(1);
            });
    const auto t0 = std::chrono::steady_clock::now();
    while (done.load() < (int)th.size()) {
        std::this_thread::sleep_for(std::chrono::milliseconds(20));
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(600)) {
            std::fprintf(stderr, "watchdog: launch did not finish (%d of %zu warps done)\n", done.load(), th.size());
            std::fflush(stderr);
            std::_Exit(3);
        }
    }
    for (auto& x : th) x.join();
    if (don) {
        // every visit ended and every slot given back
        for (int h = 0; h < kDonSlots; ++h)
            if (don->visits[h] || don->busy[h]) {
                std::printf("donation slot %d left with %u visits, busy %u\n", h, don->visits[h], don->busy[h]);
                ++failures;
                break;
            }
        if (don->held) {
            std::printf("donation slots still counted as held: %u\n", don->held);
            ++failures;
        }
    }
    delete don;
    for (int w = 0; w < warps; ++w) {
        int* base = scratch.data() + (size_t)w * per_warp;
        for (int s = 0; s < nslots; ++s)
            ASAN_UNPOISON_MEMORY_REGION(base + (size_t)s * cap + (cap - kGuard), kGuard * 4);
        ASAN_UNPOISON_MEMORY_REGION(base + (size_t)nslots * cap, kGuard * 4);
    }
    for (unsigned w : bitmaps)
        if (w) {
            std::printf("bitmap left dirty after the launch\n");
            ++failures;
            break;
        }
    for (unsigned w : dense)
        if (w) {
            std::printf("dense counters or locks left dirty after the launch\n");
            ++failures;
            break;
        }
    if (g_check[0]) {
        std::fprintf(stderr, "internal check %llu: %lld %lld %lld %lld %lld %lld\n", g_check[0], (long long)g_check[1],
                     (long long)g_check[2], (long long)g_check[3], (long long)g_check[4], (long long)g_check[5],
                     (long long)g_check[6]);
        std::_Exit(4);
    }
    std::vector<__int128> raw(n);
    for (int i = 0; i < n; ++i) raw[i] = (__int128)(((unsigned __int128)out[2 * i + 1] << 64) | out[2 * i]);
    return raw;
}

void expect_oracle(const char* what, const Csr& g, const std::vector<Sched>& ss, const Knobs& k) {
    const std::vector<__int128> raw = launch(g, ss, k);
    for (size_t i = 0; i < ss.size(); ++i) {
        uint64_t o[2];
        if (oracle_pattern_matching(g.v, g.rp.data(), g.col.data(), ss[i].tables.data(), (int)ss[i].tables.size(), 0,
                                    o))
            std::abort();
        const unsigned __int128 want = ((unsigned __int128)o[1] << 64) | o[0];
        // the host divides the raw sum by the redundancy as the reference does
        // (for label-sensitive plans the reference's raw sum is not a multiple)
        const unsigned __int128 got = (unsigned __int128)(raw[i] / (__int128)ss[i].plan.redundancy);
        if (got != want) {
            std::printf("MISMATCH %s pair %zu: got %llu want %llu (split %d leaf %d pair %d)\n", what, i,
                        (unsigned long long)got, (unsigned long long)want, k.split, k.leaf, k.pair);
            ++failures;
        }
    }
    std::printf("ok %s split=%d leaf=%d pair=%d blocks=%d wpb=%d: %zu pairs\n", what, k.split, k.leaf, k.pair, k.blocks,
                k.wpb, ss.size());
    std::fflush(stdout);
}

void case_donation() {
    const Csr g = rmat(8, 12, 31);
    std::vector<Sched> ss = motif_schedules(g, 5, true, 2);
    for (const Sched& s : motif_schedules(g, 4, true, 1)) ss.push_back(s);
    for (const Sched& s : motif_schedules(g, 5, false, 5)) ss.push_back(s);
    for (int split : {0, 1, 3})
        for (int leaf : {0, 1}) {
            Knobs k;
            k.split = split;
            k.leaf = leaf;
            expect_oracle("rmat8", g, ss, k);
        }
    const Csr h = chung_lu(200, 8.0, 2.1, 60, 9);
    std::vector<Sched> s6 = motif_schedules(h, 6, true, 13);
    Knobs k;
    k.split = 1;
    expect_oracle("chung_lu_200 six-vertex", h, s6, k);
}

// the 128-bit window merge in every merge (alpha large: merges preferred)
void case_vec() {
    const Csr g = rmat(7, 10, 33);
    std::vector<Sched> ss = motif_schedules(g, 5, true, 2);
    for (const Sched& s : motif_schedules(g, 4, false, 1)) ss.push_back(s);
    const int saved = c_merge_vec;
    c_merge_vec = 1;
    // the default weight (4) runs in every other case; here every merge
    for (int a : {1 << 20}) {
        c_merge_alpha4[0] = c_merge_alpha4[1] = c_merge_alpha4[2] = a;
        Knobs k;
        k.split = 1;
        k.leaf = 0;
        expect_oracle("rmat8 vector merge", g, ss, k);
    }
    c_merge_alpha4[0] = c_merge_alpha4[1] = c_merge_alpha4[2] = 4;
    c_merge_vec = 0;  // and the 32-wide merge on the same plans
    {
        Knobs k;
        k.split = 1;
        k.leaf = 0;
        expect_oracle("rmat7 scalar merge", g, ss, k);
    }
    c_merge_vec = saved;
}

// small enough for the CPU test suite: every path that donation touches
void case_quick() {
    const Csr g = rmat(7, 8, 31);
    std::vector<Sched> ss = motif_schedules(g, 5, true, 3);
    for (const Sched& s : motif_schedules(g, 4, true, 2)) ss.push_back(s);
    for (const Sched& s : motif_schedules(g, 5, false, 7)) ss.push_back(s);
    for (int leaf : {0, 1}) {
        Knobs k;
        k.split = 1;
        k.leaf = leaf;
        expect_oracle("rmat7", g, ss, k);
    }
    Knobs k;  // leaf bitmaps for every fixed set that does not fit the stage
    k.split = 1;
    k.stage_cap = 8;
    k.bm_min = 1;
    expect_oracle("rmat7 bitmaps", g, ss, k);
}

// hub leaf levels longer than one slice: batched leaves taken in pieces
void case_leafslices() {
    const Csr g = rmat(8, 12, 31);
    std::vector<Sched> ss = motif_schedules(g, 5, true, 3);
    Knobs k;
    k.split = 1;
    k.leaf = 1;
    expect_oracle("rmat8 leaf slices", g, ss, k);
    k.bm_min = 16;
    expect_oracle("rmat8 leaf slices + bitmaps", g, ss, k);
}

void case_pair() {
    const Csr g = chung_lu(250, 6.0, 2.5, 40, 12);
    std::vector<Sched> ss;
    for (const Sched& s : motif_schedules(g, 5, true, 1))
        if (s.plan.pair_ok) ss.push_back(s);
    if (ss.empty()) {
        std::printf("no pair-sum plan\n");
        ++failures;
        return;
    }
    for (int split : {0, 1})
        for (int log2 : {13, 5}) {  // a table that holds every task, and one that forces the fallback
            for (int dense : {0, 2}) {  // the fallback: loops, or dense counter arrays
                Knobs k;
                k.pair = 1;
                k.split = split;
                k.pair_log2 = log2;
                k.dense = dense;
                expect_oracle("pair-sum", g, ss, k);
            }
        }
}

// hubs: candidate lists of hundreds of vertices, so that the list lengths
// are computed as a shared phase and the element phases run in many slices
// of a few units each
void case_pairhub() {
    const Csr g = chung_lu(600, 8.0, 2.1, 250, 14);
    std::vector<Sched> ss;
    for (const Sched& s : motif_schedules(g, 5, true, 1))
        if (s.plan.pair_ok) ss.push_back(s);
    if (ss.empty()) {
        std::printf("no pair-sum plan\n");
        ++failures;
        return;
    }
    for (int log2 : {13, 6}) {  // the hash table, and dense arrays for the big sums
        Knobs k;
        k.pair = 1;
        k.split = 1;
        k.pair_log2 = log2;
        k.dense = 2;
        expect_oracle("pair-sum hubs", g, ss, k);
    }
}

// pair-sum tables kept across launches: entries of earlier launches carry
// older tags and are never read as live
void case_pairtags() {
    const Csr g = chung_lu(600, 8.0, 2.1, 250, 14);
    std::vector<Sched> ss;
    for (const Sched& s : motif_schedules(g, 5, true, 1))
        if (s.plan.pair_ok) ss.push_back(s);
    std::vector<unsigned long long> keep;
    for (int rep = 0; rep < 2; ++rep) {  // the second launch reuses the first's tables and tags
        Knobs k;
        k.pair = 1;
        k.split = rep == 1 ? 0 : 1;
        k.pair_log2 = 13;
        k.dense = 2;
        k.keep_tables = &keep;
        expect_oracle("pair-sum, tables kept across launches", g, ss, k);
    }
}

// The upload kernels' row search (csr_rows.cuh) on one emulated warp:
// chunks of positions as validate_kernel and relabel_fill_kernel take them,
// on CSRs with long runs of empty rows and with hubs, against each
// position's true row.
void case_rows() {
    unsigned long long state = 88172645463325252ull;
    auto rnd = [&](unsigned long long m) {
        state ^= state << 13;
        state ^= state >> 7;
        state ^= state << 17;
        return state % m;
    };
    int bad = 0, graphs = 0;
    for (int trial = 0; trial < 60; ++trial) {
        const int V = 1 + (int)rnd(2500);
        std::vector<unsigned> rp(V + 1, 0);
        for (int v = 0; v < V; ++v) {
            unsigned d = (unsigned)rnd(6);
            if (trial % 3 == 0 && rnd(10) < 9) d = 0;   // long runs of empty rows
            if (trial % 5 == 0 && rnd(500) == 0) d = 200 + (unsigned)rnd(1500);  // hubs
            rp[v + 1] = rp[v] + d;
        }
        const unsigned long long E = rp[V];
        std::vector<int> truth(E);
        for (int v = 0; v < V; ++v)
            for (unsigned k = rp[v]; k < rp[v + 1]; ++k) truth[k] = v;
        const unsigned long long chunk = trial % 2 ? 4096 : 32 + rnd(200);
        gpm_emu::block_dim = {32, 1, 1};
        gpm_emu::grid_dim = {1, 1, 1};
        std::vector<unsigned char> smem(16);
        gpm_emu::Warp* w = new gpm_emu::Warp();
        for (int l = 0; l < 32; ++l) {
            w->th[l].tid = {(unsigned)l, 0, 0};
            w->th[l].bid = {0, 0, 0};
            w->th[l].smem = smem.data();
        }
        std::atomic<int> wrong{0};
        auto body = [&](int) {
            const int lane = (int)(threadIdx.x & 31);
            for (unsigned long long c0 = 0; c0 < E; c0 += chunk) {
                const unsigned long long c1 = std::min(E, c0 + chunk);
                int r0 = 0;
                if (lane == 0) r0 = csr_row_of(rp.data(), V, c0);
                r0 = __shfl_sync(kFull, r0, 0);
                for (unsigned long long kb = c0; kb < c1; kb += 32) {
                    const int row = csr_batch_row(rp.data(), V, kb, c1, r0, lane);
                    const unsigned long long k = kb + (unsigned long long)lane;
                    if (k < c1 && row != truth[k]) wrong.fetch_add(1);
                }
            }
        };
        gpm_emu::run_warp(*w, body);
        delete w;
        bad += wrong.load();
        ++graphs;
    }
    if (bad) {
        std::printf("MISMATCH rows: %d positions got the wrong row\n", bad);
        ++failures;
    }
    std::printf("ok rows: %d CSRs\n", graphs);
}

void case_stripes() {
    const Csr g = rmat(8, 10, 8);
    std::vector<Sched> ss = motif_schedules(g, 4, true, 1);
    std::vector<__int128> first;
    for (int chunk : {1, 3, 8}) {
        Knobs k;
        k.chunk = chunk;
        k.stripes = 4;
        k.stripe = 1;
        k.split = 2;
        const std::vector<__int128> r = launch(g, ss, k);
        if (first.empty()) first = r;
        else if (r != first) {
            std::printf("MISMATCH stripes: chunk %d changes the stripe's sums\n", chunk);
            ++failures;
        }
    }
    // the stripes of a job (one per rank, say) add up to the whole job
    Knobs all;
    all.split = 2;
    const std::vector<__int128> whole = launch(g, ss, all);
    std::vector<__int128> sum(ss.size(), 0);
    for (unsigned long long st = 0; st < 4; ++st) {
        Knobs k;
        k.split = 2;
        k.stripes = 4;
        k.stripe = st;
        const std::vector<__int128> r = launch(g, ss, k);
        for (size_t i = 0; i < r.size(); ++i) sum[i] += r[i];
    }
    if (sum != whole) {
        std::printf("MISMATCH stripes: the four stripes do not add up to the whole job\n");
        ++failures;
    }
    std::printf("ok stripes\n");
}

}  // namespace

int main(int argc, char** argv) {
    std::vector<std::string> cases;
    for (int i = 1; i < argc; ++i) cases.push_back(argv[i]);
    if (cases.empty()) cases = {"quick", "pair", "pairhub", "pairtags", "stripes", "vec", "rows"};
    for (const std::string& c : cases) {
        if (c == "quick") case_quick();
        else if (c == "donation") case_donation();
        else if (c == "leafslices") case_leafslices();
        else if (c == "pair") case_pair();
        else if (c == "pairhub") case_pairhub();
        else if (c == "pairtags") case_pairtags();
        else if (c == "rows") case_rows();
        else if (c == "stripes") case_stripes();
        else if (c == "vec") case_vec();
        else {
            std::fprintf(stderr, "unknown case %s\n", c.c_str());
            return 2;
        }
    }
    std::printf("%s (%d mismatches)\n", failures ? "FAILED" : "PASSED", failures);
    return failures ? 1 : 0;
}
