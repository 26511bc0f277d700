// Schedule compiler (host).  Restates the reference's schedule construction
// so the GPU enumerator receives identical tables:
//   loop-order search and scoring ........ src/schedule.cpp:9-253
//   prefix tree ........................... src/schedule.cpp:329-362
//   restriction lists ..................... src/schedule.cpp:364-398
//   automorphisms / restriction generation  src/schedule.cpp:405-750
//   inclusion–exclusion tables ............ src/schedule.cpp:1114-1210
//   restriction validation on K_{n+1} ..... src/schedule.cpp:1433-1456
//   cost models ........................... src/schedule.cpp:1487-1713
//   redundancy calibration on K_n ......... src/schedule.cpp:1746-1764
// Floating-point cost arithmetic keeps the reference's operation order; the
// library is compiled with -ffp-contract=off so the choice does not change
// between x86 and Arm hosts.
#include "graphpi/schedule.h"
#include "gpm_internal.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>

namespace {

using PairList = std::vector<std::pair<int, int> >;

// All permutations of 0..n-1 in lexicographic order.
std::vector<std::vector<int> > all_permutations(int n) {
    std::vector<std::vector<int> > out;
    std::vector<int> p(n);
    std::iota(p.begin(), p.end(), 0);
    do out.push_back(p);
    while (std::next_permutation(p.begin(), p.end()));
    return out;
}

// Matrix of the pattern seen in loop order `order`: new vertex a is old
// vertex order[a].
std::vector<int> reorder(const int* adj, int n, const std::vector<int>& order) {
    std::vector<int> out((size_t)n * n);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) out[INDEX(a, b, n)] = adj[INDEX(order[a], order[b], n)];
    return out;
}

// Fraction of permutations that satisfy each restriction given all earlier
// ones (restrictions sorted), as used by the three cost models.
std::vector<double> restriction_ratios(int n, PairList restricts) {
    std::sort(restricts.begin(), restricts.end());
    const int r = (int)restricts.size();
    std::vector<double> sum(r, 0.0);
    std::vector<int> t(n);
    std::iota(t.begin(), t.end(), 0);
    do {
        for (int i = 0; i < r; ++i) {
            if (t[restricts[i].first] > t[restricts[i].second]) sum[i] += 1;
            else break;
        }
    } while (std::next_permutation(t.begin(), t.end()));
    double total = 1;
    for (int i = 2; i <= n; ++i) total *= i;
    for (int i = 0; i < r; ++i) sum[i] = sum[i] / total;
    for (int i = r - 1; i > 0; --i) sum[i] /= sum[i - 1];
    return sum;
}

// Depth-first search over restriction choices (reference
// aggressive_optimize_dfs, src/schedule.cpp:552-602): drop automorphisms that
// the chosen pairs already exclude; when only the identity is left, record
// the pair list; otherwise branch on each 2-cycle of the first permutation
// group that has one.
void restriction_dfs(Pattern base_dag, std::vector<std::vector<int> > iso,
                     std::vector<std::vector<std::vector<int> > > groups, PairList pairs,
                     std::vector<PairList>& out) {
    for (size_t i = 0; i < iso.size();) {
        Pattern test(base_dag);
        for (const auto& pr : pairs) test.add_ordered_edge(iso[i][pr.first], iso[i][pr.second]);
        if (!test.is_dag()) {
            groups.erase(groups.begin() + i);
            iso.erase(iso.begin() + i);
        } else {
            ++i;
        }
    }
    if (iso.size() == 1) {
        out.push_back(pairs);
        return;
    }
    for (size_t i = 0; i < groups.size();) {
        int two_cycles = 0;
        for (const auto& cyc : groups[i]) {
            if (cyc.size() != 2) continue;
            ++two_cycles;
            auto g2 = groups;
            auto i2 = iso;
            auto p2 = pairs;
            Pattern d2(base_dag);
            g2.erase(g2.begin() + i);
            i2.erase(i2.begin() + i);
            p2.push_back(std::make_pair(cyc[0], cyc[1]));
            d2.add_ordered_edge(cyc[0], cyc[1]);
            restriction_dfs(d2, i2, g2, p2, out);
        }
        if (two_cycles >= 1) break;
        ++i;
    }
}

// Removes permutation groups made of one transposition and fixed points,
// recording that transposition as a restriction (first phase of the
// reference's aggressive_optimize, src/schedule.cpp:413-440).
void take_single_transpositions(std::vector<std::vector<int> >& iso,
                                std::vector<std::vector<std::vector<int> > >& groups, PairList& pairs) {
    for (size_t i = 0; i < groups.size();) {
        int two = 0;
        std::pair<int, int> found(0, 0);
        for (const auto& cyc : groups[i]) {
            if (cyc.size() == 2) {
                ++two;
                found = std::make_pair(cyc[0], cyc[1]);
            } else if (cyc.size() != 1) {
                two = -1;
                break;
            }
        }
        if (two == 1) {
            groups.erase(groups.begin() + i);
            iso.erase(iso.begin() + i);
            pairs.push_back(found);
        } else {
            ++i;
        }
    }
}

// Counts connected spanning edge subsets of K_n by parity of their size:
// parity[0] = even, parity[1] = odd (src/schedule.cpp:1125-1155).
void connected_subsets_by_parity(int n, long long parity[2]) {
    parity[0] = parity[1] = 0;
    if (n == 1) {
        parity[0] = 1;
        return;
    }
    std::vector<std::pair<int, int> > edges;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < i; ++j) edges.push_back(std::make_pair(i, j));
    const int m = (int)edges.size();
    std::vector<int> root(n);
    for (long long s = 0; s < (1LL << m); ++s) {
        std::iota(root.begin(), root.end(), 0);
        auto find = [&](int a) {
            while (root[a] != a) a = root[a] = root[root[a]];
            return a;
        };
        int comps = n, bits = 0;
        for (int e = 0; e < m; ++e) {
            if (!(s >> e & 1)) continue;
            ++bits;
            int a = find(edges[e].first), b = find(edges[e].second);
            if (a != b) {
                root[a] = b;
                --comps;
            }
        }
        if (comps == 1) ++parity[bits & 1];
    }
}

}  // namespace

// ---------------------------------------------------------------------------

void Schedule::init_tables() {
    int max_prefix = std::max(1, size * (size - 1) / 2);
    father_prefix_id.assign(max_prefix, -1);
    last.assign(size, -1);
    next.assign(max_prefix, -1);
    loop_set_prefix_id.assign(size, -1);
    prefix.assign(max_prefix, std::vector<int>());
    restrict_last.assign(size, -1);
    restrict_next.assign(max_prefix, -1);
    restrict_index.assign(max_prefix, -1);
    total_prefix_num = 0;
    total_restrict_num = 0;
}

bool Schedule::order_is_connected() const {
    for (int i = 1; i < size; ++i) {
        bool ok = false;
        for (int j = 0; j < i && !ok; ++j) ok = adj_mat[INDEX(i, j, size)] != 0;
        if (!ok) return false;
    }
    return true;
}

Schedule::Schedule(const Pattern& pattern, bool& is_pattern_valid, int performance_modeling_type,
                   int restricts_type, bool use_in_exclusion_optimize, int v_cnt, unsigned int e_cnt,
                   long long tri_cnt) {
    if (performance_modeling_type != 0 && tri_cnt == -1)
        throw std::invalid_argument(
            "Schedule: performance modeling needs the triangle count of the data graph (tri_cnt == -1)");
    if (pattern.get_size() < 1 || pattern.get_size() > 8)
        throw std::invalid_argument("Schedule: pattern size must be in 1..8");
    is_pattern_valid = true;
    size = pattern.get_size();
    const int n = size;
    adj_mat.assign(pattern.get_adj_mat_ptr(), pattern.get_adj_mat_ptr() + n * n);

    PairList best_pairs;
    if (performance_modeling_type != 0) {
        std::vector<std::vector<int> > candidates = all_permutations(n);
        remove_invalid_permutation(candidates);
        if (performance_modeling_type == 1) {
            // keep only the orders with the longest inclusion–exclusion tail
            int best_k = 0;
            for (const auto& c : candidates) best_k = std::max(best_k, get_vec_optimize_num(c));
            std::vector<std::vector<int> > kept;
            for (const auto& c : candidates)
                if (get_vec_optimize_num(c) == best_k) kept.push_back(c);
            candidates.swap(kept);
        }
        std::vector<int> best_order(n);
        std::iota(best_order.begin(), best_order.end(), 0);
        bool have_best = false;
        double min_val = 0;
        auto score = [&](const std::vector<int>& order, const PairList& pairs) {
            if (performance_modeling_type == 1) return our_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt, tri_cnt);
            if (performance_modeling_type == 2) return GraphZero_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt);
            return Naive_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt);
        };
        // The restriction options of every order (in parallel); an order
        // with none is scored once without restrictions.
        std::vector<std::vector<PairList> > opts(candidates.size());
#pragma omp parallel for schedule(dynamic, 1)
        for (long i = 0; i < (long)candidates.size(); ++i) {
            std::vector<int> cur = reorder(pattern.get_adj_mat_ptr(), n, candidates[i]);
            if (restricts_type == 1) {
                restricts_generate(cur.data(), opts[i]);
            } else {
                Schedule probe(cur.data(), n);
                PairList pairs;
                probe.GraphZero_aggressive_optimize(pairs);
                opts[i].push_back(pairs);
            }
            if (opts[i].empty()) opts[i].push_back(PairList());
        }
        // Every candidate scored: on the GPU (one thread per candidate,
        // explicitly rounded arithmetic in the host order, so the values are
        // the host's bit for bit) when a device is present and the
        // "schedule_gpu" option is on, else on the host cores.
        std::vector<long> first(candidates.size() + 1, 0);
        for (size_t i = 0; i < candidates.size(); ++i) first[i + 1] = first[i] + (long)opts[i].size();
        std::vector<double> vals((size_t)first.back());
        bool scored = false;
#ifndef GPM_HOST_ONLY  // builds without the CUDA translation units score on the host
        if (gpm::options().schedule_gpu) {
            std::vector<int> mats, cand_order, npairs, flat;
            for (size_t i = 0; i < candidates.size(); ++i) {
                std::vector<int> cur = reorder(pattern.get_adj_mat_ptr(), n, candidates[i]);
                mats.insert(mats.end(), cur.begin(), cur.end());
                for (const auto& pairs : opts[i]) {
                    PairList sorted = pairs;
                    std::sort(sorted.begin(), sorted.end());
                    cand_order.push_back((int)i);
                    npairs.push_back((int)sorted.size());
                    for (int q = 0; q < 28; ++q) {
                        flat.push_back(q < (int)sorted.size() ? sorted[q].first : 0);
                        flat.push_back(q < (int)sorted.size() ? sorted[q].second : 0);
                    }
                }
            }
            const bool fits = npairs.empty() || *std::max_element(npairs.begin(), npairs.end()) <= 28;
            const int rc = fits ? gpm::score_candidates_gpu(n, performance_modeling_type, get_max_degree(), mats,
                                                            cand_order, npairs, flat, v_cnt, e_cnt, tri_cnt, vals)
                                : GPM_ERR_UNSUPPORTED;
            if (rc == GPM_OK) scored = true;
            else if (rc != GPM_ERR_NO_DEVICE && rc != GPM_ERR_UNSUPPORTED)
                throw std::runtime_error(std::string("Schedule: ") + gpm_last_error());
        }
#endif
        if (!scored) {
#pragma omp parallel for schedule(dynamic, 1)
            for (long i = 0; i < (long)candidates.size(); ++i)
                for (size_t j = 0; j < opts[i].size(); ++j) vals[first[i] + j] = score(candidates[i], opts[i][j]);
        }
        // the reference's sequential choice: the first strict minimum in order
        std::vector<double> order_val(candidates.size());
        std::vector<PairList> order_pairs(candidates.size());
        for (size_t i = 0; i < candidates.size(); ++i) {
            bool have = false;
            for (size_t j = 0; j < opts[i].size(); ++j) {
                const double val = vals[first[i] + j];
                if (!have || val < order_val[i]) {
                    have = true;
                    order_val[i] = val;
                    order_pairs[i] = opts[i][j];
                }
            }
        }
        for (size_t i = 0; i < candidates.size(); ++i) {
            if (!have_best || order_val[i] < min_val) {
                have_best = true;
                min_val = order_val[i];
                best_order = candidates[i];
                best_pairs = order_pairs[i];
            }
        }
        adj_mat = reorder(pattern.get_adj_mat_ptr(), n, best_order);
    } else if (restricts_type != 0) {
        std::vector<int> identity(n);
        std::iota(identity.begin(), identity.end(), 0);
        if (!order_is_connected()) {
            // the reference aborts here (its restriction generator asserts on
            // a disconnected loop order); report an invalid pattern instead
            is_pattern_valid = false;
            init_tables();
            return;
        }
        std::vector<PairList> options;
        if (restricts_type == 1) {
            restricts_generate(adj_mat.data(), options);
        } else {
            PairList pairs;
            GraphZero_aggressive_optimize(pairs);
            options.push_back(pairs);
        }
        bool have_best = false;
        double min_val = 0;
        for (const auto& pairs : options) {
            double val = restricts_type == 1 ? our_estimate_schedule_restrict(identity, pairs, v_cnt, e_cnt, tri_cnt)
                                             : GraphZero_estimate_schedule_restrict(identity, pairs, v_cnt, e_cnt);
            if (!have_best || val < min_val) {
                have_best = true;
                min_val = val;
                best_pairs = pairs;
            }
        }
    }

    if (use_in_exclusion_optimize) {
        std::vector<int> identity(n);
        std::iota(identity.begin(), identity.end(), 0);
        in_exclusion_optimize_num = get_vec_optimize_num(identity);
        if (in_exclusion_optimize_num <= 1) in_exclusion_optimize_num = 0;
        else init_in_exclusion_optimize();
    } else {
        in_exclusion_optimize_num = 0;
    }

    init_tables();
    if (!order_is_connected()) {
        is_pattern_valid = false;
        return;
    }
    build_loop_invariant();
    if (restricts_type != 0) add_restrict(best_pairs);
    set_in_exclusion_optimize_redundancy();
}

Schedule::Schedule(const Pattern& pattern, const std::vector<int>& order, const PairList& pairs,
                   bool use_in_exclusion_optimize, int restricts_type, bool& is_pattern_valid) {
    const int n = pattern.get_size();
    if (n < 1 || n > 8 || (int)order.size() != n)
        throw std::invalid_argument("Schedule: order must be a permutation of the pattern's vertices");
    std::vector<int> seen(n, 0);
    for (int x : order) {
        if (x < 0 || x >= n || seen[x]++) throw std::invalid_argument("Schedule: order is not a permutation");
    }
    for (const auto& pr : pairs)
        if (pr.first < 0 || pr.first >= n || pr.second < 0 || pr.second >= n || pr.first >= pr.second)
            throw std::invalid_argument("Schedule: restriction pairs must satisfy 0 <= first < second < n");
    size = n;
    is_pattern_valid = true;
    adj_mat = reorder(pattern.get_adj_mat_ptr(), n, order);
    if (use_in_exclusion_optimize) {
        std::vector<int> identity(n);
        std::iota(identity.begin(), identity.end(), 0);
        in_exclusion_optimize_num = get_vec_optimize_num(identity);
        if (in_exclusion_optimize_num <= 1) in_exclusion_optimize_num = 0;
        else init_in_exclusion_optimize();
    } else {
        in_exclusion_optimize_num = 0;
    }
    init_tables();
    if (!order_is_connected()) {
        is_pattern_valid = false;
        return;
    }
    build_loop_invariant();
    if (restricts_type != 0) add_restrict(pairs);
    set_in_exclusion_optimize_redundancy();
}

std::vector<Schedule::Candidate> Schedule::candidates(const Pattern& pattern, int perf, int restricts_type, int v_cnt,
                                                      unsigned int e_cnt, long long tri_cnt) {
    // the scan of the 8-argument constructor (src/schedule.cpp:30-139)
    const int n = pattern.get_size();
    std::vector<Candidate> out;
    Schedule probe;  // the pattern as given, no tables
    probe.size = n;
    probe.adj_mat.assign(pattern.get_adj_mat_ptr(), pattern.get_adj_mat_ptr() + n * n);
    std::vector<std::vector<int> > cands = all_permutations(n);
    probe.remove_invalid_permutation(cands);
    if (perf == 1) {
        int best_k = 0;
        for (const auto& c : cands) best_k = std::max(best_k, probe.get_vec_optimize_num(c));
        std::vector<std::vector<int> > kept;
        for (const auto& c : cands)
            if (probe.get_vec_optimize_num(c) == best_k) kept.push_back(c);
        cands.swap(kept);
    }
    auto score = [&](const std::vector<int>& order, const PairList& pairs) {
        if (perf == 2) return probe.GraphZero_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt);
        if (perf == 3) return probe.Naive_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt);
        return probe.our_estimate_schedule_restrict(order, pairs, v_cnt, e_cnt, tri_cnt);
    };
    // orders scored in parallel, listed in the reference's order
    std::vector<std::vector<Candidate> > per(cands.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (long i = 0; i < (long)cands.size(); ++i) {
        const std::vector<int>& order = cands[i];
        std::vector<int> cur = reorder(pattern.get_adj_mat_ptr(), n, order);
        std::vector<PairList> options;
        if (restricts_type == 1) {
            probe.restricts_generate(cur.data(), options);
        } else {
            Schedule s(cur.data(), n);
            PairList pairs;
            s.GraphZero_aggressive_optimize(pairs);
            options.push_back(pairs);
        }
        if (options.empty()) options.push_back(PairList());
        for (const auto& pairs : options) per[i].push_back(Candidate{order, pairs, score(order, pairs)});
    }
    for (auto& v : per) out.insert(out.end(), v.begin(), v.end());
    return out;
}

Schedule::Schedule(const int* adj, int n) {
    if (n < 1 || n > 8) throw std::invalid_argument("Schedule: pattern size must be in 1..8");
    size = n;
    adj_mat.assign(adj, adj + n * n);
    in_exclusion_optimize_num = 0;
    init_tables();
    if (!order_is_connected()) throw std::invalid_argument("Schedule: invalid schedule (loop order not connected)");
    build_loop_invariant();
    set_in_exclusion_optimize_redundancy();
}

Schedule::~Schedule() {}

int Schedule::get_max_degree() const {
    int best = 0;
    for (int i = 0; i < size; ++i) {
        int d = 0;
        for (int j = 0; j < size; ++j) d += adj_mat[INDEX(i, j, size)];
        best = std::max(best, d);
    }
    return best;
}

void Schedule::build_loop_invariant() {
    loop_set_prefix_id[0] = -1;
    std::vector<int> members;
    for (int i = 1; i < size; ++i) {
        members.clear();
        for (int j = 0; j < i; ++j)
            if (adj_mat[INDEX(i, j, size)]) members.push_back(j);
        loop_set_prefix_id[i] = find_father_prefix((int)members.size(), members.data());
    }
}

int Schedule::find_father_prefix(int data_size, const int* data) {
    if (data_size == 0) return -1;
    const int tail = data[data_size - 1];
    for (int id = last[tail]; id != -1; id = next[id])
        if ((int)prefix[id].size() == data_size && std::equal(data, data + data_size, prefix[id].begin())) return id;
    const int father = find_father_prefix(data_size - 1, data);
    const int id = total_prefix_num++;
    father_prefix_id[id] = father;
    next[id] = last[tail];
    last[tail] = id;
    prefix[id].assign(data, data + data_size);
    return id;
}

void Schedule::add_restrict(const std::vector<std::pair<int, int> >& restricts) {
    // drop pairs implied by two others: (a, c) when (a, b) and (b, c) exist
    restrict_pair = restricts;
    for (size_t i = 0; i < restrict_pair.size();) {
        bool keep = true;
        for (size_t j = 0; j < restrict_pair.size() && keep; ++j) {
            if (i == j || restrict_pair[j].first != restrict_pair[i].first) continue;
            for (size_t k = 0; k < restrict_pair.size(); ++k)
                if (i != k && j != k && restrict_pair[k].second == restrict_pair[i].second &&
                    restrict_pair[j].second == restrict_pair[k].first) {
                    keep = false;
                    break;
                }
        }
        if (keep) ++i;
        else restrict_pair.erase(restrict_pair.begin() + i);
    }
    std::fill(restrict_last.begin(), restrict_last.end(), -1);
    std::fill(restrict_next.begin(), restrict_next.end(), -1);
    total_restrict_num = 0;
    for (const auto& p : restrict_pair) {
        // at loop depth p.second the vertex id must stay below chosen[p.first]
        restrict_index[total_restrict_num] = p.first;
        restrict_next[total_restrict_num] = restrict_last[p.second];
        restrict_last[p.second] = total_restrict_num;
        ++total_restrict_num;
    }
}

int Schedule::get_multiplicity() const { return (int)get_isomorphism_vec().size(); }

std::vector<std::vector<int> > Schedule::get_isomorphism_vec() const {
    std::vector<std::vector<int> > out;
    for (const auto& v : all_permutations(size)) {
        bool ok = true;
        for (int i = 0; i < size && ok; ++i)
            for (int j = i + 1; j < size; ++j)
                if (adj_mat[INDEX(i, j, size)] && !adj_mat[INDEX(v[i], v[j], size)]) {
                    ok = false;
                    break;
                }
        if (ok) out.push_back(v);
    }
    return out;
}

std::vector<std::vector<int> > Schedule::calc_permutation_group(const std::vector<int> vec, int size) {
    std::vector<char> used(size, 0);
    std::vector<std::vector<int> > cycles;
    for (size_t i = 0; i < vec.size(); ++i) {
        if (used[i]) continue;
        std::vector<int> cyc{(int)i};
        used[i] = 1;
        for (int x = vec[i]; !used[x]; x = vec[x]) {
            used[x] = 1;
            cyc.push_back(x);
        }
        cycles.push_back(cyc);
    }
    return cycles;
}

void Schedule::aggressive_optimize(std::vector<std::pair<int, int> >& ordered_pairs) const {
    auto iso = get_isomorphism_vec();
    std::vector<std::vector<std::vector<int> > > groups;
    for (const auto& v : iso) groups.push_back(calc_permutation_group(v, size));
    ordered_pairs.clear();
    take_single_transpositions(iso, groups, ordered_pairs);
    Pattern base_dag(size);
    for (const auto& p : ordered_pairs) base_dag.add_ordered_edge(p.first, p.second);
    bool changed = true;
    while (changed && iso.size() != 1) {
        for (size_t i = 0; i < iso.size();) {
            Pattern test(base_dag);
            for (const auto& p : ordered_pairs) test.add_ordered_edge(iso[i][p.first], iso[i][p.second]);
            if (!test.is_dag()) {
                groups.erase(groups.begin() + i);
                iso.erase(iso.begin() + i);
            } else {
                ++i;
            }
        }
        changed = false;
        for (size_t i = 0; i < groups.size();) {
            const std::vector<int>* two = nullptr;
            for (const auto& cyc : groups[i])
                if (cyc.size() == 2) {
                    two = &cyc;
                    break;
                }
            if (two) {
                std::pair<int, int> found((*two)[0], (*two)[1]);
                groups.erase(groups.begin() + i);
                iso.erase(iso.begin() + i);
                ordered_pairs.push_back(found);
                base_dag.add_ordered_edge(found.first, found.second);
                changed = true;
                break;
            }
            ++i;
        }
    }
}

void Schedule::aggressive_optimize_get_all_pairs(std::vector<std::vector<std::pair<int, int> > >& ordered_pairs_vector) {
    auto iso = get_isomorphism_vec();
    std::vector<std::vector<std::vector<int> > > groups;
    for (const auto& v : iso) groups.push_back(calc_permutation_group(v, size));
    ordered_pairs_vector.clear();
    PairList pairs;
    take_single_transpositions(iso, groups, pairs);
    Pattern base_dag(size);
    for (const auto& p : pairs) base_dag.add_ordered_edge(p.first, p.second);
    restriction_dfs(base_dag, iso, groups, pairs, ordered_pairs_vector);
}

// Orderings of n distinct values that satisfy every pair (value[second] <
// value[first]): a subset DP that assigns the values from the smallest up.
static long long linear_extensions(int n, const std::vector<std::pair<int, int> >& pairs) {
    unsigned below[8] = {0};
    for (const auto& p : pairs) below[p.first] |= 1u << p.second;
    std::vector<long long> ways((size_t)1 << n, 0);
    ways[0] = 1;
    for (unsigned mask = 0; mask < (1u << n); ++mask) {
        if (!ways[mask]) continue;
        for (int v = 0; v < n; ++v)
            if (!(mask >> v & 1) && (below[v] & ~mask) == 0) ways[mask | (1u << v)] += ways[mask];
    }
    return ways[((size_t)1 << n) - 1];
}

// Keeps the restriction sets under which the pattern is counted exactly once
// per embedding.  The reference decides it by counting on the complete graph
// K_{n+1} with and without the set (src/schedule.cpp:1433-1456).  On a
// complete graph every injective map is an embedding, so those counts are
// (n+1)! / |Aut| (all maps, one per automorphism class) and (n+1) x the
// number of orderings of n values the set allows: the test is exactly
// linear_extensions(set) x |Aut| == n!, decided here without enumerating.
void Schedule::restricts_generate(const int* cur_adj_mat, std::vector<std::vector<std::pair<int, int> > >& restricts) {
    Schedule base(cur_adj_mat, size);
    base.aggressive_optimize_get_all_pairs(restricts);
    const int n = base.get_size();
    long long fact = 1;
    for (int i = 2; i <= n; ++i) fact *= i;
    const long long aut = base.get_multiplicity();
    for (size_t i = 0; i < restricts.size();) {
        if (linear_extensions(n, restricts[i]) * aut != fact) restricts.erase(restricts.begin() + i);
        else ++i;
    }
}

void Schedule::GraphZero_get_automorphisms(std::vector<std::vector<int> >& Aut) const {
    Aut.clear();
    for (const auto& p : all_permutations(size)) {
        bool ok = true;
        for (int i = 0; i < size && ok; ++i)
            for (int j = 0; j < size; ++j)
                if (adj_mat[INDEX(i, j, size)] != adj_mat[INDEX(p[i], p[j], size)]) {
                    ok = false;
                    break;
                }
        if (ok) Aut.push_back(p);
    }
}

void Schedule::GraphZero_aggressive_optimize(std::vector<std::pair<int, int> >& ordered_pairs) const {
    std::vector<std::vector<int> > aut;
    GraphZero_get_automorphisms(aut);
    PairList L;
    for (int v = 0; v < size; ++v) {
        std::vector<std::vector<int> > stabilizer;
        for (const auto& x : aut) {
            if (x[v] == v) {
                stabilizer.push_back(x);
                continue;
            }
            std::pair<int, int> cur(std::min(v, x[v]), std::max(v, x[v]));
            if (std::find(L.begin(), L.end(), cur) == L.end()) L.push_back(cur);
        }
        aut.swap(stabilizer);
    }
    ordered_pairs.clear();
    for (const auto& l : L) {
        bool fresh = true;
        for (auto& p : ordered_pairs)
            if (l.second == p.second) {
                fresh = false;
                if (l.first > p.first) p.first = l.first;
                break;
            }
        if (fresh) ordered_pairs.push_back(l);
    }
}

int Schedule::get_vec_optimize_num(const std::vector<int>& vec) const {
    for (int i = 1; i < size; ++i) {
        bool linked = false;
        for (int j = 0; j < i && !linked; ++j) linked = adj_mat[INDEX(vec[i], vec[j], size)] != 0;
        if (!linked) return -1;
    }
    // the longest tail of mutually non-adjacent loops
    for (int k = 2; k <= size; ++k)
        for (int i = size - k + 1; i < size; ++i)
            if (adj_mat[INDEX(vec[size - k], vec[i], size)]) return k - 1;
    return size;  // only reachable for a pattern without edges
}

void Schedule::remove_invalid_permutation(std::vector<std::vector<int> >& candidates) const {
    std::vector<std::vector<int> > kept;
    for (const auto& vec : candidates) {
        bool ok = true;
        for (int x = 1; x < size && ok; ++x) {
            bool linked = false;
            for (int y = 0; y < x && !linked; ++y) linked = adj_mat[INDEX(vec[x], vec[y], size)] != 0;
            ok = linked;
        }
        if (ok) kept.push_back(vec);
    }
    candidates.swap(kept);
}

int Schedule::get_in_exclusion_optimize_num_when_not_optimize() {
    std::vector<int> identity(size);
    std::iota(identity.begin(), identity.end(), 0);
    return get_vec_optimize_num(identity);
}

double Schedule::our_estimate_schedule_restrict(const std::vector<int>& order, const PairList& pairs, int v_cnt,
                                                unsigned int e_cnt, long long tri_cnt) const {
    const int n = size;
    const int md = std::max(2, get_max_degree());
    std::vector<double> p_size(md), pp_size(md);
    const double p0 = e_cnt * 1.0 / v_cnt / v_cnt;
    const double p1 = tri_cnt * 1.0 * v_cnt / e_cnt / e_cnt;
    p_size[0] = v_cnt;
    for (int i = 1; i < md; ++i) p_size[i] = p_size[i - 1] * p0;
    pp_size[0] = 1;
    for (int i = 1; i < md; ++i) pp_size[i] = pp_size[i - 1] * p1;

    std::vector<int> cur = reorder(adj_mat.data(), n, order);
    PairList restricts = pairs;
    std::sort(restricts.begin(), restricts.end());
    std::vector<double> ratio = restriction_ratios(n, restricts);

    std::vector<std::vector<int> > invariant(n);
    double val = 1;
    for (int i = n - 1; i >= 0; --i) {
        int forward = 0;
        for (int j = 0; j < i; ++j) forward += cur[INDEX(j, i, n)] ? 1 : 0;
        int c = forward;
        for (int j = i - 1; j >= 0; --j)
            if (cur[INDEX(j, i, n)]) invariant[j].push_back(c--);
        for (int x : invariant[i])
            if (x > 1) val += p_size[1] * pp_size[x - 2] + p_size[1];
        val += 1;
        for (size_t j = 0; j < restricts.size(); ++j)
            if (restricts[j].second == i) val *= ratio[j];
        if (i) val *= p_size[1] * pp_size[forward - 1];
        else val *= p_size[0];
    }
    return val;
}

double Schedule::GraphZero_estimate_schedule_restrict(const std::vector<int>& order, const PairList& pairs, int v_cnt,
                                                      unsigned int e_cnt) const {
    const int n = size;
    // one more entry than the reference allocates: its p_size[max_degree]
    // read (when a vertex has max_degree earlier neighbours) is past the end
    const int md = std::max(2, get_max_degree()) + 1;
    std::vector<double> p_size(md);
    const double p = e_cnt * 1.0 / v_cnt / v_cnt;
    p_size[0] = v_cnt;
    for (int i = 1; i < md; ++i) p_size[i] = p_size[i - 1] * p;

    std::vector<int> cur = reorder(adj_mat.data(), n, order);
    PairList restricts = pairs;
    std::sort(restricts.begin(), restricts.end());
    std::vector<double> ratio = restriction_ratios(n, restricts);

    std::vector<std::vector<int> > invariant(n);
    double val = 1;
    for (int i = n - 1; i >= 0; --i) {
        int forward = 0;
        for (int j = 0; j < i; ++j) forward += cur[INDEX(j, i, n)] ? 1 : 0;
        int c = forward;
        for (int j = i - 1; j >= 0; --j)
            if (cur[INDEX(j, i, n)]) invariant[j].push_back(c--);
        for (int x : invariant[i])
            if (x > 1) val += p_size[x - 1] + p_size[1];
        for (size_t j = 0; j < restricts.size(); ++j)
            if (restricts[j].second == i) val *= ratio[j];
        val *= p_size[forward];
    }
    return val;
}

double Schedule::Naive_estimate_schedule_restrict(const std::vector<int>& order, const PairList& pairs, int v_cnt,
                                                  unsigned int e_cnt) const {
    const int n = size;
    const double p = e_cnt * 2.0 / v_cnt / v_cnt;
    std::vector<int> cur = reorder(adj_mat.data(), n, order);
    PairList restricts = pairs;
    std::sort(restricts.begin(), restricts.end());
    std::vector<double> ratio = restriction_ratios(n, restricts);
    double val = 1;
    for (int i = n - 1; i >= 0; --i) {
        int forward = 0;
        for (int j = 0; j < i; ++j) forward += cur[INDEX(j, i, n)] ? 1 : 0;
        for (size_t j = 0; j < restricts.size(); ++j)
            if (restricts[j].second == i) val *= ratio[j];
        val *= v_cnt;
        for (int j = 0; j < i - forward; ++j) val *= (1 - p);
        for (int j = 0; j < forward; ++j) val *= p;
    }
    return val;
}

void Schedule::init_in_exclusion_optimize() {
    const int k = in_exclusion_optimize_num;
    // e_minus_o[s] = (#even - #odd) connected spanning edge subsets of K_s
    std::vector<long long> even(k + 1), odd(k + 1);
    for (int s = 1; s <= k; ++s) {
        long long par[2];
        connected_subsets_by_parity(s, par);
        even[s] = par[0];
        odd[s] = par[1];
    }
    in_exclusion_optimize_group.clear();
    in_exclusion_optimize_val.clear();
    // Enumerate set partitions of {0..k-1} as restricted-growth strings,
    // "open a new block" before "join block 0, 1, ..." at every position.
    std::vector<int> block_of(k, 0);
    struct Walker {
        Schedule* self;
        int k;
        std::vector<int>& block_of;
        const std::vector<long long>& even;
        const std::vector<long long>& odd;
        void emit(int blocks) {
            std::vector<int> bsize(blocks, 0);
            for (int i = 0; i < k; ++i) ++bsize[block_of[i]];
            long long v0 = even[bsize[0]], v1 = odd[bsize[0]];
            for (int b = 1; b < blocks; ++b) {
                long long t0 = v0, t1 = v1;
                v0 = t0 * even[bsize[b]] + t1 * odd[bsize[b]];
                v1 = t0 * odd[bsize[b]] + t1 * even[bsize[b]];
            }
            std::vector<std::vector<int> > group(blocks);
            for (int i = 0; i < k; ++i) group[block_of[i]].push_back(i);
            self->in_exclusion_optimize_group.push_back(group);
            self->in_exclusion_optimize_val.push_back((int)(v0 - v1));
        }
        void walk(int depth, int blocks) {
            if (depth == k) {
                emit(blocks);
                return;
            }
            block_of[depth] = blocks;
            walk(depth + 1, blocks + 1);
            for (int b = 0; b < blocks; ++b) {
                block_of[depth] = b;
                walk(depth + 1, blocks);
            }
        }
    };
    Walker w{this, k, block_of, even, odd};
    w.walk(0, 0);
}

void Schedule::set_in_exclusion_optimize_redundancy() {
    const int k = in_exclusion_optimize_num;
    if (k <= 1) {
        in_exclusion_optimize_redundancy = 1;
        return;
    }
    in_exclusion_optimize_redundancy = 1;
    long long with_iep = complete_graph_count(*this, size);
    in_exclusion_optimize_num = 0;
    long long without = complete_graph_count(*this, size);
    in_exclusion_optimize_num = k;
    in_exclusion_optimize_redundancy = with_iep / without;
}

void Schedule::print_schedule() const {
    printf("Schedule:\n");
    for (int i = 0; i < size; ++i) {
        for (int j = 0; j < size; ++j) printf("%d", adj_mat[INDEX(i, j, size)]);
        puts("");
    }
}

std::vector<int64_t> Schedule::pack() const {
    std::vector<int64_t> v;
    const int n = size, P = total_prefix_num, R = total_restrict_num;
    v.push_back(n);
    for (int i = 0; i < n * n; ++i) v.push_back(adj_mat[i]);
    v.push_back(P);
    for (int i = 0; i < P; ++i) v.push_back(father_prefix_id[i]);
    for (int i = 0; i < n; ++i) v.push_back(last[i]);
    for (int i = 0; i < P; ++i) v.push_back(next[i]);
    for (int i = 0; i < n; ++i) v.push_back(loop_set_prefix_id[i]);
    v.push_back(R);
    for (int i = 0; i < n; ++i) v.push_back(restrict_last[i]);
    for (int i = 0; i < R; ++i) v.push_back(restrict_next[i]);
    for (int i = 0; i < R; ++i) v.push_back(restrict_index[i]);
    v.push_back((int64_t)restrict_pair.size());
    for (const auto& p : restrict_pair) {
        v.push_back(p.first);
        v.push_back(p.second);
    }
    v.push_back(in_exclusion_optimize_num);
    v.push_back((int64_t)in_exclusion_optimize_group.size());
    for (size_t g = 0; g < in_exclusion_optimize_group.size(); ++g) {
        v.push_back(in_exclusion_optimize_val[g]);
        v.push_back((int64_t)in_exclusion_optimize_group[g].size());
        for (const auto& blk : in_exclusion_optimize_group[g]) {
            v.push_back((int64_t)blk.size());
            for (int x : blk) v.push_back(x);
        }
    }
    v.push_back(in_exclusion_optimize_redundancy);
    v.push_back(get_multiplicity());
    return v;
}

// ---------------------------------------------------------------------------
// Nested-loop count on K_m (schedule construction only).

namespace {

struct CompleteCounter {
    const Schedule& s;
    int n, m, k;
    std::vector<std::vector<int> > sets;  // per prefix id
    std::vector<int> chosen;
    long long ans = 0;

    CompleteCounter(const Schedule& sch, int m_) : s(sch), n(sch.get_size()), m(m_), k(sch.get_in_exclusion_optimize_num()) {
        sets.resize(std::max(1, s.get_total_prefix_num()));
    }
    // N(v) in K_m
    void neighbours(int v, std::vector<int>& out) const {
        out.clear();
        for (int u = 0; u < m; ++u)
            if (u != v) out.push_back(u);
    }
    void build(int prefix_id, int v) {
        int father = s.get_father_prefix_id(prefix_id);
        std::vector<int> nb;
        neighbours(v, nb);
        if (father == -1) {
            sets[prefix_id] = nb;
            return;
        }
        std::vector<int> out;
        std::set_intersection(sets[father].begin(), sets[father].end(), nb.begin(), nb.end(), std::back_inserter(out));
        sets[prefix_id] = out;
    }
    long long outside_chosen(const std::vector<int>& S, size_t len) const {
        long long r = (long long)len;
        for (int c : chosen)
            if (std::binary_search(S.begin(), S.begin() + len, c)) --r;
        return r;
    }
    int bound(int depth) const {
        int mv = m;
        for (int i = s.get_restrict_last(depth); i != -1; i = s.get_restrict_next(i))
            mv = std::min(mv, chosen[s.get_restrict_index(i)]);
        return mv;
    }
    void run(int depth) {
        const std::vector<int>& S = sets[s.get_loop_set_prefix_id(depth)];
        if (S.empty()) return;
        if (depth == n - k) {
            for (size_t g = 0; g < s.in_exclusion_optimize_group.size(); ++g) {
                long long val = s.in_exclusion_optimize_val[g];
                for (const auto& blk : s.in_exclusion_optimize_group[g]) {
                    std::vector<int> acc = sets[s.get_loop_set_prefix_id(depth + blk[0])];
                    for (size_t b = 1; b < blk.size(); ++b) {
                        const auto& other = sets[s.get_loop_set_prefix_id(depth + blk[b])];
                        std::vector<int> t;
                        std::set_intersection(acc.begin(), acc.end(), other.begin(), other.end(), std::back_inserter(t));
                        acc.swap(t);
                    }
                    val *= outside_chosen(acc, acc.size());
                    if (val == 0) break;
                }
                ans += val;
            }
            return;
        }
        if (depth == n - 1) {
            if (s.get_total_restrict_num() > 0) {
                size_t len = std::lower_bound(S.begin(), S.end(), bound(depth)) - S.begin();
                if (len > 0) ans += outside_chosen(S, len);
            } else {
                ans += outside_chosen(S, S.size());
            }
            return;
        }
        const int mv = bound(depth);
        const std::vector<int> loop = S;  // chain builds below never touch S
        for (int v : loop) {
            if (mv <= v) break;
            if (std::find(chosen.begin(), chosen.end(), v) != chosen.end()) continue;
            bool empty = false;
            for (int p = s.get_last(depth); p != -1; p = s.get_next(p)) {
                build(p, v);
                if (sets[p].empty()) {
                    empty = true;
                    break;
                }
            }
            if (empty) continue;
            chosen.push_back(v);
            run(depth + 1);
            chosen.pop_back();
        }
    }
};

}  // namespace

long long complete_graph_count(const Schedule& schedule, int m) {
    if (schedule.get_size() < 2 || m < 1) return 0;
    CompleteCounter c(schedule, m);
    for (int v = 0; v < m; ++v) {
        for (int p = schedule.get_last(0); p != -1; p = schedule.get_next(p)) c.build(p, v);
        c.chosen.push_back(v);
        c.run(1);
        c.chosen.pop_back();
    }
    return c.ans / schedule.get_in_exclusion_optimize_redundancy();
}
