// Host half of the C ABI: options, motif generation, the schedule
// compiler entry point, and decoding schedule tables into a device plan.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <exception>
#include <map>
#include <mutex>
#include <string>

#include "gpm_internal.h"
#include "graphpi/motif_generator.h"
#include "graphpi/schedule.h"

namespace gpm {

Options& options() {
    static Options o;
    return o;
}

namespace {

struct Reader {
    const int64_t* t;
    int32_t n, pos = 0;
    bool ok = true;
    int64_t get() {
        if (pos >= n) {
            ok = false;
            return 0;
        }
        return t[pos++];
    }
};

}  // namespace

int compile_plan(const int64_t* t, int32_t n_words, DevPlan* out) {
    if (!t || n_words <= 0 || !out) {
        set_error("gpm_plan_create: empty tables");
        return GPM_ERR_INVALID_ARG;
    }
    Reader r{t, n_words};
    DevPlan p;
    memset(&p, 0, sizeof p);
    const int n = (int)r.get();
    if (n < 2 || n > kMaxN) {
        set_error("gpm_plan_create: pattern size %d outside 2..%d", n, kMaxN);
        return GPM_ERR_UNSUPPORTED;
    }
    p.n = n;
    for (int i = 0; i < n * n; ++i) r.get();  // adjacency: not needed by the kernels
    const int P = (int)r.get();
    if (P < 1 || P > kMaxPrefix) {
        set_error("gpm_plan_create: %d prefixes outside 1..%d", P, kMaxPrefix);
        return GPM_ERR_INVALID_ARG;
    }
    p.nprefix = P;
    int father[kMaxPrefix], last[kMaxN], next[kMaxPrefix];
    for (int i = 0; i < P; ++i) father[i] = (int)r.get();
    for (int i = 0; i < n; ++i) last[i] = (int)r.get();
    for (int i = 0; i < P; ++i) next[i] = (int)r.get();
    for (int i = 0; i < n; ++i) p.loop_set[i] = (int)r.get();
    const int R = (int)r.get();
    if (R < 0 || R > kMaxPrefix) {
        set_error("gpm_plan_create: %d restrictions outside 0..%d", R, kMaxPrefix);
        return GPM_ERR_INVALID_ARG;
    }
    int rlast[kMaxN], rnext[kMaxPrefix], rindex[kMaxPrefix];
    for (int i = 0; i < n; ++i) rlast[i] = (int)r.get();
    for (int i = 0; i < R; ++i) rnext[i] = (int)r.get();
    for (int i = 0; i < R; ++i) rindex[i] = (int)r.get();
    const int npairs = (int)r.get();
    if (npairs < 0 || npairs > 64) {
        set_error("gpm_plan_create: bad restriction pair count %d", npairs);
        return GPM_ERR_INVALID_ARG;
    }
    for (int i = 0; i < 2 * npairs; ++i) r.get();
    const int k = (int)r.get();
    const int ngroups = (int)r.get();
    if (!r.ok) {
        set_error("gpm_plan_create: tables truncated");
        return GPM_ERR_INVALID_ARG;
    }
    // --- validate the tree ---
    for (int i = 0; i < P; ++i) {
        if (father[i] < -1 || father[i] >= i || next[i] < -1 || next[i] >= P) {
            set_error("gpm_plan_create: malformed prefix table at %d", i);
            return GPM_ERR_INVALID_ARG;
        }
    }
    for (int d = 0; d < n; ++d) {
        if (last[d] < -1 || last[d] >= P || rlast[d] < -1 || rlast[d] >= R) {
            set_error("gpm_plan_create: malformed depth table at %d", d);
            return GPM_ERR_INVALID_ARG;
        }
        if (d >= 1 && (p.loop_set[d] < 0 || p.loop_set[d] >= P)) {
            set_error("gpm_plan_create: depth %d has no loop set", d);
            return GPM_ERR_INVALID_ARG;
        }
    }
    if (k != 0 && (k < 2 || k > n - 1 || k > 6)) {
        set_error("gpm_plan_create: inclusion-exclusion length %d unsupported", k);
        return GPM_ERR_UNSUPPORTED;
    }
    p.k = k;
    p.T = k ? n - k : n - 1;
    p.L = p.T - 1;
    // chains: prefixes whose last member is depth d, in the reference's order
    int cnt = 0;
    for (int d = 0; d < n; ++d) {
        p.chain_begin[d] = cnt;
        int guard = 0;
        for (int id = last[d]; id != -1; id = next[id]) {
            if (cnt >= kMaxPrefix || ++guard > P) {
                set_error("gpm_plan_create: cyclic prefix chain at depth %d", d);
                return GPM_ERR_INVALID_ARG;
            }
            p.chain_list[cnt++] = id;
        }
    }
    p.chain_begin[n] = cnt;
    // restriction masks
    for (int d = 0; d < n; ++d) {
        unsigned m = 0;
        int guard = 0;
        for (int i = rlast[d]; i != -1; i = rnext[i]) {
            if (i < 0 || i >= R || ++guard > R) {
                set_error("gpm_plan_create: malformed restriction list at depth %d", d);
                return GPM_ERR_INVALID_ARG;
            }
            if (rindex[i] < 0 || rindex[i] >= d) {
                set_error("gpm_plan_create: restriction at depth %d names depth %d", d, rindex[i]);
                return GPM_ERR_INVALID_ARG;
            }
            m |= 1u << rindex[i];
        }
        p.rmask[d] = m;
    }
    // scratch slots
    int slots = 0;
    for (int i = 0; i < P; ++i) {
        p.father[i] = father[i];
        p.slot[i] = father[i] >= 0 ? slots++ : -1;
    }
    p.nslots = slots + 2;
    // count-only fusion: without a tail, the prefix built at level L is the
    // last loop's set and nothing else reads it
    p.count_only = -1;
    if (k == 0 && p.L >= 0) {
        int b = p.chain_begin[p.L], e = p.chain_begin[p.L + 1];
        if (e - b == 1 && p.chain_list[b] == p.loop_set[p.T] && father[p.chain_list[b]] >= 0)
            p.count_only = p.chain_list[b];
    }
    // inclusion–exclusion groups; singleton blocks get ids 0..k-1
    p.nblocks = k;
    for (int i = 0; i < k; ++i) p.block_mask[i] = 1u << i;
    if (ngroups < 0 || ngroups > kMaxGroups) {
        set_error("gpm_plan_create: %d inclusion-exclusion groups exceed %d", ngroups, kMaxGroups);
        return GPM_ERR_UNSUPPORTED;
    }
    p.ngroups = ngroups;
    int entries = 0;
    for (int g = 0; g < ngroups; ++g) {
        p.group_coef[g] = (int)r.get();
        p.group_begin[g] = entries;
        const int nb = (int)r.get();
        if (nb < 1 || nb > k) {
            set_error("gpm_plan_create: malformed inclusion-exclusion group %d", g);
            return GPM_ERR_INVALID_ARG;
        }
        for (int b = 0; b < nb; ++b) {
            const int len = (int)r.get();
            if (len < 1 || len > k) {
                set_error("gpm_plan_create: malformed block in group %d", g);
                return GPM_ERR_INVALID_ARG;
            }
            unsigned mask = 0;
            for (int j = 0; j < len; ++j) {
                int m = (int)r.get();
                if (m < 0 || m >= k) {
                    set_error("gpm_plan_create: block member %d out of range", m);
                    return GPM_ERR_INVALID_ARG;
                }
                mask |= 1u << m;
            }
            int id = -1;
            for (int q = 0; q < p.nblocks; ++q)
                if (p.block_mask[q] == mask) id = q;
            if (id < 0) {
                if (p.nblocks >= kMaxBlocks) {
                    set_error("gpm_plan_create: too many inclusion-exclusion blocks");
                    return GPM_ERR_UNSUPPORTED;
                }
                id = p.nblocks++;
                p.block_mask[id] = mask;
            }
            if (entries >= kMaxGroupEntries) {
                set_error("gpm_plan_create: inclusion-exclusion table too large");
                return GPM_ERR_UNSUPPORTED;
            }
            p.group_block[entries++] = (unsigned char)id;
        }
    }
    p.group_begin[ngroups] = entries;
    p.redundancy = r.get();
    if (!r.ok || p.redundancy < 1) {
        set_error("gpm_plan_create: tables truncated or redundancy < 1");
        return GPM_ERR_INVALID_ARG;
    }
    if (k && ngroups == 0) {
        set_error("gpm_plan_create: inclusion-exclusion length %d without groups", k);
        return GPM_ERR_INVALID_ARG;
    }
    p.label_sensitive = plan_label_sensitive(p);
    // ---- leaf batching of the deepest loop level L (L >= 2) ----
    p.leaf_kind = kLeafGeneric;
    p.leaf_fa = p.leaf_fb = p.leaf_sa = p.leaf_sb = -1;
    p.leaf_ka = p.leaf_kb = 0;
    p.leaf_cab = p.leaf_cx = 0;
    // depth at which a prefix is built = its last member = the depth of the chain holding it
    int built_at[kMaxPrefix];
    for (int d = 0; d < n; ++d)
        for (int c = p.chain_begin[d]; c < p.chain_begin[d + 1]; ++c) built_at[p.chain_list[c]] = d;
    if (p.L >= 2) {
        if (k == 0) {
            const int st = p.loop_set[p.T];
            if (built_at[st] == p.L) {
                p.leaf_kind = kLeafCount;
                p.leaf_fa = father[st];  // -1: the set is N(v) itself
                const int L1 = p.L - 1, f = father[st];
                const bool f_is_nbr = f >= 0 && father[f] < 0 && built_at[f] == L1 &&
                                      p.chain_begin[L1 + 1] - p.chain_begin[L1] == 1;
                const bool b_fixed = built_at[p.loop_set[p.L]] < L1 && !((p.rmask[p.L] >> L1) & 1u);
                const bool t_fixed = (p.rmask[p.T] >> L1) == 0;
                p.pair_ok = (L1 >= 2 && f_is_nbr && b_fixed && t_fixed) ? 1 : 0;
            }
        } else if (k == 2 && ngroups == 2) {
            // groups {a}{b} and {a,b} in either order
            int gab = -1, gx = -1;
            for (int g = 0; g < 2; ++g) {
                const int nb = p.group_begin[g + 1] - p.group_begin[g];
                if (nb == 2) gab = g;
                if (nb == 1 && p.block_mask[p.group_block[p.group_begin[g]]] == 3u) gx = g;
            }
            // every set built at L must be one of the two tail sets
            bool only_tail_sets = true;
            for (int c = p.chain_begin[p.L]; c < p.chain_begin[p.L + 1]; ++c)
                only_tail_sets &= p.chain_list[c] == p.loop_set[p.T] || p.chain_list[c] == p.loop_set[p.T + 1];
            if (gab >= 0 && gx >= 0 && only_tail_sets) {
                p.leaf_kind = kLeafIep2;
                p.leaf_cab = p.group_coef[gab];
                p.leaf_cx = p.group_coef[gx];
                p.leaf_sa = p.loop_set[p.T];
                p.leaf_sb = p.loop_set[p.T + 1];
                int* kinds[2] = {&p.leaf_ka, &p.leaf_kb};
                int* probes[2] = {&p.leaf_fa, &p.leaf_fb};
                const int ids[2] = {p.leaf_sa, p.leaf_sb};
                for (int q = 0; q < 2; ++q) {
                    const int sid = ids[q];
                    if (built_at[sid] < p.L) {
                        *kinds[q] = 0;  // fixed: probe is the set itself
                        *probes[q] = sid;
                    } else if (father[sid] < 0) {
                        *kinds[q] = 1;  // N(v)
                        *probes[q] = -1;
                    } else {
                        *kinds[q] = 2;  // father ∩ N(v)
                        *probes[q] = father[sid];
                    }
                }
            }
        }
    }
    *out = p;
    return GPM_OK;
}

// ---------------------------------------------------------------------------
// Host model of the enumeration.  The reference's inclusion–exclusion tail
// skips the restrictions of its own loops and divides by a redundancy
// measured on K_n (src/graph.cpp:306-344, src/schedule.cpp:1746-1764).
// When a skipped restriction ties a tail loop to an earlier loop, the
// overcount differs from prefix to prefix and the reference's result depends
// on the vertex labels (some 6-vertex patterns, e.g. K3,3 and the hourglass,
// are off from the true count).  Such plans must see the caller's labels to
// reproduce the reference's output; the check below counts each plan on
// small random graphs under several labellings.

namespace {

struct ProbeDfs {
    const DevPlan& p;
    int V;
    const std::vector<uint32_t>& rp;
    const std::vector<int32_t>& col;
    std::vector<std::vector<int> > sets;
    int chosen[kMaxN];
    __int128 acc = 0;

    ProbeDfs(const DevPlan& plan, int v, const std::vector<uint32_t>& r, const std::vector<int32_t>& c)
        : p(plan), V(v), rp(r), col(c), sets(kMaxPrefix) {}

    std::vector<int> nbr(int v) const { return std::vector<int>(col.begin() + rp[v], col.begin() + rp[v + 1]); }

    int bound(int d) const {
        int b = V;
        for (int j = 0; j < d; ++j)
            if (p.rmask[d] >> j & 1) b = std::min(b, chosen[j]);
        return b;
    }

    long long outside(const std::vector<int>& S, size_t len, int nch) const {
        long long r = (long long)len;
        for (int j = 0; j < nch; ++j)
            if (std::binary_search(S.begin(), S.begin() + len, chosen[j])) --r;
        return r;
    }

    bool build(int d, int v) {
        std::vector<int> nv = nbr(v);
        for (int c = p.chain_begin[d]; c < p.chain_begin[d + 1]; ++c) {
            const int pid = p.chain_list[c], f = p.father[pid];
            if (f < 0) {
                sets[pid] = nv;
            } else {
                std::vector<int> o;
                std::set_intersection(sets[f].begin(), sets[f].end(), nv.begin(), nv.end(), std::back_inserter(o));
                sets[pid].swap(o);
            }
            if (sets[pid].empty()) return false;
        }
        return true;
    }

    __int128 tail() {
        const int T = p.T;
        const std::vector<int>& S = sets[p.loop_set[T]];
        if (S.empty()) return 0;
        if (!p.k) {
            size_t lb = std::lower_bound(S.begin(), S.end(), bound(T)) - S.begin();
            return outside(S, lb, T);
        }
        long long bv[kMaxBlocks];
        for (int b = 0; b < p.nblocks; ++b) {
            std::vector<int> a;
            bool first = true;
            for (int i = 0; i < p.k; ++i) {
                if (!(p.block_mask[b] >> i & 1)) continue;
                const std::vector<int>& Si = sets[p.loop_set[T + i]];
                if (first) {
                    a = Si;
                    first = false;
                } else {
                    std::vector<int> o;
                    std::set_intersection(a.begin(), a.end(), Si.begin(), Si.end(), std::back_inserter(o));
                    a.swap(o);
                }
            }
            bv[b] = outside(a, a.size(), T);
        }
        __int128 total = 0;
        for (int g = 0; g < p.ngroups; ++g) {
            __int128 v = p.group_coef[g];
            for (int q = p.group_begin[g]; q < p.group_begin[g + 1]; ++q) v *= bv[p.group_block[q]];
            total += v;
        }
        return total;
    }

    void level(int d) {
        if (d == p.T) {
            acc += tail();
            return;
        }
        const std::vector<int> S = sets[p.loop_set[d]];
        const int b = bound(d);
        for (int v : S) {
            if (v >= b) break;
            bool dup = false;
            for (int j = 0; j < d; ++j) dup |= chosen[j] == v;
            if (dup || !build(d, v)) continue;
            chosen[d] = v;
            level(d + 1);
        }
    }
};

// Erdős–Rényi graph from a fixed seed, relabelled by perm.
void probe_graph(int n, double prob, uint64_t seed, const std::vector<int>& perm, std::vector<uint32_t>& rp,
                 std::vector<int32_t>& col) {
    std::vector<std::vector<int> > adj(n);
    uint64_t x = seed;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            x = x * 6364136223846793005ull + 1442695040888963407ull;
            if ((double)(x >> 11) / 9007199254740992.0 < prob) {
                adj[perm[i]].push_back(perm[j]);
                adj[perm[j]].push_back(perm[i]);
            }
        }
    rp.assign(n + 1, 0);
    col.clear();
    for (int i = 0; i < n; ++i) {
        std::sort(adj[i].begin(), adj[i].end());
        col.insert(col.end(), adj[i].begin(), adj[i].end());
        rp[i + 1] = (uint32_t)col.size();
    }
}

}  // namespace

__int128 plan_probe_count(const DevPlan& p, int v_cnt, const std::vector<uint32_t>& rowptr,
                          const std::vector<int32_t>& col) {
    ProbeDfs dfs(p, v_cnt, rowptr, col);
    for (int v = 0; v < v_cnt; ++v) {
        dfs.chosen[0] = v;
        if (!dfs.build(0, v)) continue;
        dfs.level(1);
    }
    return dfs.acc;
}

int plan_label_sensitive(const DevPlan& p) {
    // without skipped restrictions every valid schedule counts exactly
    bool skipped = false;
    for (int d = p.T; d < p.n && p.k; ++d) skipped |= p.rmask[d] != 0;
    if (!skipped) return 0;
    static std::mutex mu;
    static std::map<std::string, int> memo;
    std::string key((const char*)&p, sizeof(DevPlan));
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = memo.find(key);
        if (it != memo.end()) return it->second;
    }
    int sensitive = 0;
    const int sizes[3] = {10, 12, 13};
    for (int gi = 0; gi < 3 && !sensitive; ++gi) {
        const int n = sizes[gi];
        std::vector<int> ident(n), rev(n), mix(n);
        for (int i = 0; i < n; ++i) ident[i] = i, rev[i] = n - 1 - i, mix[i] = (i * 7 + 3) % n;
        std::vector<uint32_t> rp;
        std::vector<int32_t> col;
        probe_graph(n, 0.55, 0x5eed0000ull + gi, ident, rp, col);
        const __int128 base = plan_probe_count(p, n, rp, col);
        for (const auto* perm : {&rev, &mix}) {
            probe_graph(n, 0.55, 0x5eed0000ull + gi, *perm, rp, col);
            if (plan_probe_count(p, n, rp, col) != base) sensitive = 1;
        }
    }
    std::lock_guard<std::mutex> lk(mu);
    memo[key] = sensitive;
    return sensitive;
}

}  // namespace gpm

using gpm::set_error;

extern "C" {


GPM_API int gpm_motifs(int32_t k, int32_t* adj_out, int32_t cap, int32_t* count) {
    gpm::clear_error();
    if (k < 1 || k > gpm::kMaxN || !count || (cap > 0 && !adj_out)) {
        set_error("gpm_motifs: k must be in 1..%d", gpm::kMaxN);
        return GPM_ERR_INVALID_ARG;
    }
    MotifGenerator mg(k);
    std::vector<Pattern> ps = mg.generate();
    int c = 0;
    for (const Pattern& p : ps) {
        if (c < cap) memcpy(adj_out + (size_t)c * k * k, p.get_adj_mat_ptr(), sizeof(int32_t) * k * k);
        ++c;
    }
    *count = c;
    return GPM_OK;
}

GPM_API int gpm_pattern_multiplicity(int32_t n, const int32_t* adj, int64_t* out) {
    gpm::clear_error();
    if (n < 1 || n > gpm::kMaxN || !adj || !out) {
        set_error("gpm_pattern_multiplicity: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    Pattern p(n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (adj[i * n + j]) p.add_edge(i, j);
    // multiplicity is a property of the matrix; any loop order will do
    int64_t m = 0;
    {
        std::vector<int> perm(n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        do {
            bool ok = true;
            for (int i = 0; i < n && ok; ++i)
                for (int j = i + 1; j < n; ++j)
                    if (p.get_adj_mat_ptr()[i * n + j] && !p.get_adj_mat_ptr()[perm[i] * n + perm[j]]) {
                        ok = false;
                        break;
                    }
            m += ok;
        } while (std::next_permutation(perm.begin(), perm.end()));
    }
    *out = m;
    return GPM_OK;
}

GPM_API int gpm_schedule_build(int32_t n, const int32_t* adj, int32_t perf_type, int32_t restricts_type,
                               int32_t use_iep, int64_t v_cnt, uint64_t e_cnt, int64_t tri_cnt, int64_t* tables,
                               int32_t cap, int32_t* n_words, int32_t* valid) {
    gpm::clear_error();
    if (n < 2 || n > gpm::kMaxN || !adj || !n_words || !valid) {
        set_error("gpm_schedule_build: pattern size must be in 2..%d", gpm::kMaxN);
        return GPM_ERR_INVALID_ARG;
    }
    if (perf_type < 0 || perf_type > 3 || restricts_type < 0 || restricts_type > 2) {
        set_error("gpm_schedule_build: perf_type must be 0..3 and restricts_type 0..2");
        return GPM_ERR_INVALID_ARG;
    }
    if (perf_type != 0 && tri_cnt < 0) {
        set_error("gpm_schedule_build: performance modeling needs tri_cnt >= 0");
        return GPM_ERR_INVALID_ARG;
    }
    if (v_cnt < 1 || v_cnt > INT32_MAX || e_cnt > UINT32_MAX || (perf_type != 0 && e_cnt == 0)) {
        set_error("gpm_schedule_build: v_cnt/e_cnt out of range");
        return GPM_ERR_INVALID_ARG;
    }
    try {
        Pattern p(n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                if (adj[i * n + j] != adj[j * n + i]) {
                    set_error("gpm_schedule_build: adjacency matrix is not symmetric");
                    return GPM_ERR_INVALID_ARG;
                }
                if (adj[i * n + j] && i != j) p.add_edge(i, j);
            }
        bool ok = false;
        Schedule s(p, ok, perf_type, restricts_type, use_iep != 0, (int)v_cnt, (unsigned)e_cnt, tri_cnt);
        *valid = ok ? 1 : 0;
        std::vector<int64_t> t = ok ? s.pack() : std::vector<int64_t>();
        *n_words = (int32_t)t.size();
        if ((int32_t)t.size() > cap || (!tables && !t.empty())) {
            set_error("gpm_schedule_build: output needs %d words, capacity %d", (int)t.size(), cap);
            return GPM_ERR_INVALID_ARG;
        }
        if (!t.empty()) memcpy(tables, t.data(), t.size() * sizeof(int64_t));
        return GPM_OK;
    } catch (const std::exception& e) {
        set_error("gpm_schedule_build: %s", e.what());
        return GPM_ERR_INVALID_ARG;
    }
}

GPM_API int gpm_schedule_candidates(int32_t n, const int32_t* adj, int32_t perf_type, int32_t restricts_type,
                                    int64_t v_cnt, uint64_t e_cnt, int64_t tri_cnt, int32_t* orders,
                                    int32_t* n_pairs, int32_t* pairs, double* costs, int32_t cap,
                                    int32_t* count) {
    gpm::clear_error();
    if (n < 2 || n > gpm::kMaxN || !adj || !count || cap < 0 || (cap > 0 && (!orders || !n_pairs || !pairs || !costs))) {
        set_error("gpm_schedule_candidates: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    if (perf_type < 1 || perf_type > 3 || restricts_type < 0 || restricts_type > 2 || v_cnt < 1 || e_cnt == 0 ||
        e_cnt > UINT32_MAX || (perf_type == 1 && tri_cnt < 0)) {
        set_error("gpm_schedule_candidates: perf_type must be 1..3 with valid graph statistics");
        return GPM_ERR_INVALID_ARG;
    }
    try {
        Pattern p(n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                if (adj[i * n + j] && i != j) p.add_edge(i, j);
        auto cands = Schedule::candidates(p, perf_type, restricts_type, (int)v_cnt, (unsigned)e_cnt, tri_cnt);
        *count = (int32_t)cands.size();
        for (int c = 0; c < (int)cands.size() && c < cap; ++c) {
            for (int j = 0; j < n; ++j) orders[c * n + j] = cands[c].order[j];
            const int np = std::min<int>((int)cands[c].pairs.size(), GPM_MAX_PAIRS);
            n_pairs[c] = np;
            for (int q = 0; q < np; ++q) {
                pairs[(size_t)c * 2 * GPM_MAX_PAIRS + 2 * q] = cands[c].pairs[q].first;
                pairs[(size_t)c * 2 * GPM_MAX_PAIRS + 2 * q + 1] = cands[c].pairs[q].second;
            }
            costs[c] = cands[c].cost;
        }
        return GPM_OK;
    } catch (const std::exception& e) {
        set_error("gpm_schedule_candidates: %s", e.what());
        return GPM_ERR_INVALID_ARG;
    }
}

GPM_API int gpm_schedule_from_order(int32_t n, const int32_t* adj, const int32_t* order, int32_t n_pairs,
                                    const int32_t* pairs, int32_t use_iep, int32_t restricts_type, int64_t* tables,
                                    int32_t cap, int32_t* n_words, int32_t* valid) {
    gpm::clear_error();
    if (n < 2 || n > gpm::kMaxN || !adj || !order || n_pairs < 0 || n_pairs > GPM_MAX_PAIRS ||
        (n_pairs > 0 && !pairs) || !n_words || !valid) {
        set_error("gpm_schedule_from_order: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    try {
        Pattern p(n);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                if (adj[i * n + j] && i != j) p.add_edge(i, j);
        std::vector<int> ord(order, order + n);
        std::vector<std::pair<int, int> > pr;
        for (int q = 0; q < n_pairs; ++q) pr.push_back(std::make_pair(pairs[2 * q], pairs[2 * q + 1]));
        bool ok = false;
        Schedule s(p, ord, pr, use_iep != 0, restricts_type, ok);
        *valid = ok ? 1 : 0;
        std::vector<int64_t> t = ok ? s.pack() : std::vector<int64_t>();
        *n_words = (int32_t)t.size();
        if ((int32_t)t.size() > cap || (!tables && !t.empty())) {
            set_error("gpm_schedule_from_order: output needs %d words, capacity %d", (int)t.size(), cap);
            return GPM_ERR_INVALID_ARG;
        }
        if (!t.empty()) memcpy(tables, t.data(), t.size() * sizeof(int64_t));
        return GPM_OK;
    } catch (const std::exception& e) {
        set_error("gpm_schedule_from_order: %s", e.what());
        return GPM_ERR_INVALID_ARG;
    }
}

GPM_API int gpm_schedule_analyze(const int64_t* tables, int32_t n_words, int32_t* label_sensitive) {
    gpm::clear_error();
    if (!label_sensitive) return GPM_ERR_INVALID_ARG;
    gpm::DevPlan p;
    int rc = gpm::compile_plan(tables, n_words, &p);
    if (rc) return rc;
    *label_sensitive = p.label_sensitive;
    return GPM_OK;
}

GPM_API int gpm_plan_info(const int64_t* tables, int32_t n_words, int32_t* info, int32_t cap) {
    gpm::clear_error();
    if (!info || cap < 6) {
        set_error("gpm_plan_info: need room for 6 values");
        return GPM_ERR_INVALID_ARG;
    }
    gpm::DevPlan p;
    int rc = gpm::compile_plan(tables, n_words, &p);
    if (rc) return rc;
    info[0] = p.T;
    info[1] = p.L;
    info[2] = p.k;
    info[3] = p.leaf_kind;
    info[4] = p.pair_ok;
    info[5] = p.label_sensitive;
    return GPM_OK;
}

GPM_API int gpm_set_option(const char* key, int64_t value) {
    gpm::clear_error();
    if (!key) return GPM_ERR_INVALID_ARG;
    gpm::Options& o = gpm::options();
    std::string k(key);
    int64_t* slot = nullptr;
    int64_t lo = 0, hi = INT64_MAX;
    if (k == "warps_per_block") slot = &o.warps_per_block, lo = 1, hi = 32;
    else if (k == "blocks_per_sm") slot = &o.blocks_per_sm, lo = 1, hi = 32;
    else if (k == "chunk") slot = &o.chunk, lo = 1, hi = 1 << 20;
    else if (k == "count_bytes") slot = &o.count_bytes, lo = 0, hi = 1;
    else if (k == "timeout_ms") slot = &o.timeout_ms, lo = 1, hi = 3600 * 1000;
    else if (k == "stage_max") slot = &o.stage_max, lo = 0, hi = 1 << 14;
    else if (k == "stage_tma") slot = &o.stage_tma, lo = 0, hi = 1;
    else if (k == "schedule_gpu") slot = &o.schedule_gpu, lo = 0, hi = 1;
    else if (k == "merge_vec") slot = &o.merge_vec, lo = 0, hi = 1;
    else if (k == "pool") slot = &o.pool, lo = 0, hi = 1;
    else if (k == "leaf_batch") slot = &o.leaf_batch, lo = 0, hi = 1;
    else if (k == "pair_leaf") slot = &o.pair_leaf, lo = 0, hi = 1;
    else if (k == "pair_log2") slot = &o.pair_log2, lo = 0, hi = 24;
    else if (k == "dense_slots") slot = &o.dense_slots, lo = 0, hi = 1024;
    else if (k == "pair_max_ops") slot = &o.pair_max_ops, lo = 0, hi = (int64_t)1 << 40;
    else if (k == "bitmap_min") slot = &o.bitmap_min, lo = 0, hi = 1 << 30;
    else if (k == "min_blocks") {
        if (value != 1 && value != 3 && value != 4 && value != 5) {
            set_error("gpm_set_option: min_blocks is 1, 3, 4 or 5");
            return GPM_ERR_INVALID_ARG;
        }
        slot = &o.min_blocks, lo = 1, hi = 5;
    }
    else if (k == "split") slot = &o.split, lo = 0, hi = 1 << 30;
    else if (k == "stripes") slot = &o.stripes, lo = 1, hi = 1 << 30;
    else if (k == "stripe") slot = &o.stripe, lo = 0, hi = (1 << 30) - 1;
    else if (k == "raw_sums") slot = &o.raw_sums, lo = 0, hi = 1;
    else if (k == "merge_alpha4_small") slot = &o.merge_alpha4[0], lo = 0, hi = 1024;
    else if (k == "merge_alpha4_mid") slot = &o.merge_alpha4[1], lo = 0, hi = 1024;
    else if (k == "merge_alpha4_large") slot = &o.merge_alpha4[2], lo = 0, hi = 1024;
    if (!slot) {
        set_error("gpm_set_option: unknown key '%s'", key);
        return GPM_ERR_INVALID_ARG;
    }
    if (value < lo || value > hi) {
        set_error("gpm_set_option: %s=%lld outside [%lld, %lld]", key, (long long)value, (long long)lo, (long long)hi);
        return GPM_ERR_INVALID_ARG;
    }
    *slot = value;
    return GPM_OK;
}

GPM_API int gpm_get_option(const char* key, int64_t* value) {
    gpm::clear_error();
    if (!key || !value) return GPM_ERR_INVALID_ARG;
    gpm::Options& o = gpm::options();
    std::string k(key);
    if (k == "warps_per_block") *value = o.warps_per_block;
    else if (k == "blocks_per_sm") *value = o.blocks_per_sm;
    else if (k == "chunk") *value = o.chunk;
    else if (k == "count_bytes") *value = o.count_bytes;
    else if (k == "timeout_ms") *value = o.timeout_ms;
    else if (k == "stage_max") *value = o.stage_max;
    else if (k == "stage_tma") *value = o.stage_tma;
    else if (k == "schedule_gpu") *value = o.schedule_gpu;
    else if (k == "merge_vec") *value = o.merge_vec;
    else if (k == "pool") *value = o.pool;
    else if (k == "leaf_batch") *value = o.leaf_batch;
    else if (k == "pair_leaf") *value = o.pair_leaf;
    else if (k == "pair_log2") *value = o.pair_log2;
    else if (k == "dense_slots") *value = o.dense_slots;
    else if (k == "pair_max_ops") *value = o.pair_max_ops;
    else if (k == "bitmap_min") *value = o.bitmap_min;
    else if (k == "min_blocks") *value = o.min_blocks;
    else if (k == "split") *value = o.split;
    else if (k == "stripes") *value = o.stripes;
    else if (k == "stripe") *value = o.stripe;
    else if (k == "raw_sums") *value = o.raw_sums;
    else if (k == "merge_alpha4_small") *value = o.merge_alpha4[0];
    else if (k == "merge_alpha4_mid") *value = o.merge_alpha4[1];
    else if (k == "merge_alpha4_large") *value = o.merge_alpha4[2];
    else {
        set_error("gpm_get_option: unknown key '%s'", key);
        return GPM_ERR_INVALID_ARG;
    }
    return GPM_OK;
}

}  // extern "C"
