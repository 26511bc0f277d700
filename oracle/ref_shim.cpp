// Test infrastructure only: a C-callable shim over the reference GraphPi
// library, compiled together with the reference's own sources (never copied)
// by oracle/build_ref.sh into oracle/_ref/libgraphpi_ref.so.  Only tests/ and
// the fixture generator in tests/golden/ load it, to pin the oracle against
// the reference itself.
//
// Entry points map onto the reference API:
//   ref_graph_from_csr      -> a reference `Graph` filled from our CSR (public
//                              fields, include/graph.h:9-16), with
//                              `VertexSet::max_intersection_size` set the way
//                              DataLoader does (src/dataloader.cpp:112-115)
//   ref_pattern_matching    -> Graph::pattern_matching (src/graph.cpp:199-245)
//   ref_triangle_counting_mt-> Graph::triangle_counting_mt (src/graph.cpp:112-139)
//   ref_schedule_create     -> Schedule 8-argument ctor (src/schedule.cpp:9-253)
//   ref_schedule_dump       -> the schedule getters (include/schedule.h:23-37)
//   ref_motifs              -> MotifGenerator::generate (src/motif_generator.cpp:33-43)
//   ref_load_data           -> DataLoader::load_data (src/dataloader.cpp:8-163)
//   ref_stripes_raw         -> the counting of Graph::pattern_matching split
//                              into first-level tasks (root vertices, or the
//                              directed edges (v0, v1) of the CSR) and summed
//                              per stripe t mod S == s; each task runs the
//                              reference's own root-loop body
//                              (src/graph.cpp:212-228), one depth-1 loop
//                              iteration (:366-396) and
//                              pattern_matching_aggressive_func from depth 2
//
// The depth-level function is private to Graph (include/graph.h:50-55); this
// test-only translation unit opens the class so that it can call it.  The
// reference's own objects are compiled unchanged.
#define private public
#include "graph.h"
#undef private
#include "dataloader.h"
#include "pattern.h"
#include "schedule.h"
#include "motif_generator.h"
#include "vertex_set.h"

#include <algorithm>
#include <cstring>
#include <vector>

extern "C" {

void* ref_graph_from_csr(int v_cnt, const unsigned* rowptr, const int* col, long long tri_cnt, int threads) {
    Graph* g = new Graph();
    g->v_cnt = v_cnt;
    g->e_cnt = rowptr[v_cnt];
    g->vertex = new unsigned[v_cnt + 1];
    g->edge = new int[g->e_cnt > 0 ? g->e_cnt : 1];
    memcpy(g->vertex, rowptr, sizeof(unsigned) * (v_cnt + 1));
    memcpy(g->edge, col, sizeof(int) * g->e_cnt);
    std::vector<int> deg(v_cnt);
    for (int v = 0; v < v_cnt; ++v) deg[v] = (int)(rowptr[v + 1] - rowptr[v]);
    std::sort(deg.begin(), deg.end());
    int second = v_cnt >= 2 ? deg[v_cnt - 2] : (v_cnt == 1 ? deg[0] : 0);
    VertexSet::max_intersection_size = std::max(VertexSet::max_intersection_size, second);
    g->max_degree = v_cnt >= 1 ? deg[v_cnt - 1] : 0;
    g->tri_cnt = tri_cnt >= 0 ? tri_cnt : g->triangle_counting_mt(threads);
    return g;
}

void ref_graph_free(void* g) { delete (Graph*)g; }

long long ref_graph_tri(void* g) { return ((Graph*)g)->tri_cnt; }
int ref_graph_v(void* g) { return ((Graph*)g)->v_cnt; }
unsigned ref_graph_e(void* g) { return ((Graph*)g)->e_cnt; }
int ref_graph_max_degree(void* g) { return ((Graph*)g)->max_degree; }

int ref_graph_export(void* gp, unsigned* rowptr, int* col) {
    Graph* g = (Graph*)gp;
    memcpy(rowptr, g->vertex, sizeof(unsigned) * (g->v_cnt + 1));
    memcpy(col, g->edge, sizeof(int) * g->e_cnt);
    return 0;
}

long long ref_triangle_counting_mt(void* g, int threads) { return ((Graph*)g)->triangle_counting_mt(threads); }
long long ref_triangle_counting(void* g) { return ((Graph*)g)->triangle_counting(); }

void* ref_schedule_create(int n, const int* adj, int perf, int restr, int iep,
                          int v_cnt, unsigned e_cnt, long long tri_cnt, int* valid) {
    Pattern p(n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (adj[i * n + j]) p.add_edge(i, j);
    bool ok = false;
    Schedule* s = new Schedule(p, ok, perf, restr, iep != 0, v_cnt, e_cnt, tri_cnt);
    *valid = ok ? 1 : 0;
    return s;
}

void ref_schedule_free(void* s) { delete (Schedule*)s; }

// Flattened tables, in this order:
// size, adj[n*n], total_prefix_num, father[P], last[n], next[P], loop_set[n],
// total_restrict_num, restrict_last[n], restrict_next[R], restrict_index[R],
// n_pairs, pairs[2*n_pairs], iep_num, n_groups,
//   per group: val, n_blocks, per block: len, members...,
// redundancy, multiplicity.
int ref_schedule_dump(void* sp, long long* out, int cap) {
    Schedule* s = (Schedule*)sp;
    std::vector<long long> v;
    int n = s->get_size();
    v.push_back(n);
    const int* adj = s->get_adj_mat_ptr();
    for (int i = 0; i < n * n; ++i) v.push_back(adj[i]);
    int P = s->get_total_prefix_num();
    v.push_back(P);
    for (int i = 0; i < P; ++i) v.push_back(s->get_father_prefix_id(i));
    for (int i = 0; i < n; ++i) v.push_back(s->get_last(i));
    for (int i = 0; i < P; ++i) v.push_back(s->get_next(i));
    for (int i = 0; i < n; ++i) v.push_back(s->get_loop_set_prefix_id(i));
    int R = s->get_total_restrict_num();
    v.push_back(R);
    for (int i = 0; i < n; ++i) v.push_back(s->get_restrict_last(i));
    for (int i = 0; i < R; ++i) v.push_back(s->get_restrict_next(i));
    for (int i = 0; i < R; ++i) v.push_back(s->get_restrict_index(i));
    v.push_back((long long)s->restrict_pair.size());
    for (auto& pr : s->restrict_pair) { v.push_back(pr.first); v.push_back(pr.second); }
    v.push_back(s->get_in_exclusion_optimize_num());
    v.push_back((long long)s->in_exclusion_optimize_group.size());
    for (size_t g = 0; g < s->in_exclusion_optimize_group.size(); ++g) {
        v.push_back(s->in_exclusion_optimize_val[g]);
        const auto& grp = s->in_exclusion_optimize_group[g];
        v.push_back((long long)grp.size());
        for (const auto& blk : grp) {
            v.push_back((long long)blk.size());
            for (int x : blk) v.push_back(x);
        }
    }
    v.push_back(s->get_in_exclusion_optimize_redundancy());
    v.push_back(s->get_multiplicity());
    if ((int)v.size() > cap) return -(int)v.size();
    for (size_t i = 0; i < v.size(); ++i) out[i] = v[i];
    return (int)v.size();
}

long long ref_pattern_matching(void* g, void* s, int threads) {
    return ((Graph*)g)->pattern_matching(*(Schedule*)s, threads);
}

// Writes the adjacency matrices of all connected k-vertex motifs (k*k ints
// each) in generation order and returns how many there are.
int ref_motifs(int k, int* out, int cap_patterns) {
    MotifGenerator mg(k);
    std::vector<Pattern> ps = mg.generate();
    int cnt = 0;
    for (const Pattern& p : ps) {
        if (cnt < cap_patterns) memcpy(out + (size_t)cnt * k * k, p.get_adj_mat_ptr(), sizeof(int) * k * k);
        ++cnt;
    }
    return cnt;
}

// DataLoader::load_data with the Wiki_Vote data type (tri_cnt from the
// reference's constant table).
void* ref_load_data(const char* path, int data_type, int oriented_type) {
    DataLoader D;
    Graph* g = nullptr;
    if (!D.load_data(g, (DataType)data_type, path, oriented_type)) return nullptr;
    return g;
}

// Raw (undivided) sums of one schedule over the stripes ids[0, n_ids) of
// `stripes`: out[j] = sum over the tasks t of stripe ids[j].  The tasks of
// all stripes share one dynamically scheduled loop.  Sums are the
// reference's long long; where they exceed 64 bits they wrap, so callers
// compare them modulo 2^64.
int ref_stripes_raw(void* gp, void* sp, long long stripes, const long long* ids, int n_ids, int threads,
                    long long* out) {
    Graph* g = (Graph*)gp;
    const Schedule& s = *(Schedule*)sp;
    const int n = s.get_size(), k = s.get_in_exclusion_optimize_num();
    const int T = k ? n - k : n - 1;
    const long long nt = T == 1 ? (long long)g->v_cnt : (long long)g->e_cnt;
    std::vector<long long> task;
    std::vector<int> owner;
    for (int j = 0; j < n_ids; ++j)
        for (long long t = ids[j]; t < nt; t += stripes) {
            task.push_back(t);
            owner.push_back(j);
        }
    std::vector<long long> sums(n_ids, 0);
#pragma omp parallel num_threads(threads)
    {
        VertexSet* vertex_set = new VertexSet[s.get_total_prefix_num()];
        VertexSet subtraction_set;
        VertexSet tmp_set;
        subtraction_set.init();
        std::vector<long long> mine(n_ids, 0);
#pragma omp for schedule(dynamic)
        for (long long x = 0; x < (long long)task.size(); ++x) {
            const long long t = task[x];
            long long local_ans = 0;
            int v0, v1 = -1;
            if (T == 1) {
                v0 = (int)t;
            } else {
                v0 = (int)(std::upper_bound(g->vertex, g->vertex + g->v_cnt + 1, (unsigned)t) - g->vertex) - 1;
                v1 = g->edge[t];
            }
            unsigned l, r;
            g->get_edge_index(v0, l, r);
            for (int p = s.get_last(0); p != -1; p = s.get_next(p))
                vertex_set[p].build_vertex_set(s, vertex_set, &g->edge[l], (int)r - l, p);
            subtraction_set.push_back(v0);
            if (T == 1) {
                g->pattern_matching_aggressive_func(s, vertex_set, subtraction_set, tmp_set, local_ans, 1);
            } else {
                int min_vertex = g->v_cnt;
                for (int i = s.get_restrict_last(1); i != -1; i = s.get_restrict_next(i))
                    if (min_vertex > subtraction_set.get_data(s.get_restrict_index(i)))
                        min_vertex = subtraction_set.get_data(s.get_restrict_index(i));
                if (min_vertex > v1 && !subtraction_set.has_data(v1)) {
                    g->get_edge_index(v1, l, r);
                    bool is_zero = false;
                    for (int p = s.get_last(1); p != -1; p = s.get_next(p)) {
                        vertex_set[p].build_vertex_set(s, vertex_set, &g->edge[l], (int)r - l, p, v1);
                        if (vertex_set[p].get_size() == 0) {
                            is_zero = true;
                            break;
                        }
                    }
                    if (!is_zero) {
                        subtraction_set.push_back(v1);
                        g->pattern_matching_aggressive_func(s, vertex_set, subtraction_set, tmp_set, local_ans, 2);
                        subtraction_set.pop_back();
                    }
                }
            }
            subtraction_set.pop_back();
            mine[owner[x]] += local_ans;
        }
#pragma omp critical
        for (int j = 0; j < n_ids; ++j) sums[j] += mine[j];
        delete[] vertex_set;
    }
    for (int j = 0; j < n_ids; ++j) out[j] = sums[j];
    return 0;
}

}  // extern "C"
