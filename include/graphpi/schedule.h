// Schedule — the host-side schedule compiler: loop order, symmetry-breaking
// restrictions, prefix-set tree and inclusion–exclusion tables consumed by
// the GPU enumerator.  Same public interface as the reference's Schedule
// (include/schedule.h:9-97 of thu-pacman/GraphPi); tables are identical for
// the same inputs.
#pragma once
#include <cstdint>
#include <utility>
#include <vector>
#include "pattern.h"

class Schedule {
public:
    // performance_modeling_type 0: none, 1: GraphPi model, 2: GraphZero
    // model, 3: naive model.  restricts_type 0: none, 1: GraphPi restriction
    // generator, 2: GraphZero's.  (include/schedule.h:14-20)
    Schedule(const Pattern& pattern, bool& is_pattern_valid, int performance_modeling_type,
             int restricts_type, bool use_in_exclusion_optimize, int v_cnt, unsigned int e_cnt,
             long long tri_cnt = 0);
    Schedule(const int* adj_mat, int size);
    // The schedule the constructor above would build had its cost model
    // picked `order` (new vertex i = pattern vertex order[i]) and restriction
    // set `pairs` (in the reordered numbering).  restricts_type 0 drops the
    // pairs, as the constructor does.
    Schedule(const Pattern& pattern, const std::vector<int>& order, const std::vector<std::pair<int, int> >& pairs,
             bool use_in_exclusion_optimize, int restricts_type, bool& is_pattern_valid);
    ~Schedule();

    // Every (loop order, restriction set) the constructor scores for these
    // inputs, in its scan order, with the cost its model assigns.
    struct Candidate {
        std::vector<int> order;
        std::vector<std::pair<int, int> > pairs;
        double cost;
    };
    static std::vector<Candidate> candidates(const Pattern& pattern, int performance_modeling_type, int restricts_type,
                                             int v_cnt, unsigned int e_cnt, long long tri_cnt);

    inline int get_total_prefix_num() const { return total_prefix_num; }
    inline int get_father_prefix_id(int prefix_id) const { return father_prefix_id[prefix_id]; }
    inline int get_loop_set_prefix_id(int loop) const { return loop_set_prefix_id[loop]; }
    inline int get_size() const { return size; }
    inline int get_last(int i) const { return last[i]; }
    inline int get_next(int i) const { return next[i]; }
    inline int get_in_exclusion_optimize_num() const { return in_exclusion_optimize_num; }
    inline void set_in_exclusion_optimize_num(int num) { in_exclusion_optimize_num = num; }
    int get_in_exclusion_optimize_num_when_not_optimize();
    void add_restrict(const std::vector<std::pair<int, int> >& restricts);
    inline int get_total_restrict_num() const { return total_restrict_num; }
    inline int get_restrict_last(int i) const { return restrict_last[i]; }
    inline int get_restrict_next(int i) const { return restrict_next[i]; }
    inline int get_restrict_index(int i) const { return restrict_index[i]; }
    inline long long get_in_exclusion_optimize_redundancy() const { return in_exclusion_optimize_redundancy; }
    int get_max_degree() const;
    int get_multiplicity() const;
    void aggressive_optimize(std::vector<std::pair<int, int> >& ordered_pairs) const;
    void aggressive_optimize_get_all_pairs(std::vector<std::vector<std::pair<int, int> > >& ordered_pairs_vector);
    void restricts_generate(const int* cur_adj_mat, std::vector<std::vector<std::pair<int, int> > >& restricts);
    void GraphZero_aggressive_optimize(std::vector<std::pair<int, int> >& ordered_pairs) const;
    void GraphZero_get_automorphisms(std::vector<std::vector<int> >& Aut) const;
    std::vector<std::vector<int> > get_isomorphism_vec() const;
    static std::vector<std::vector<int> > calc_permutation_group(const std::vector<int> vec, int size);
    inline const int* get_adj_mat_ptr() const { return adj_mat.data(); }
    void print_schedule() const;

    // Cost models (public here so the learned model and tests can score
    // candidate orders with them).
    double our_estimate_schedule_restrict(const std::vector<int>& order, const std::vector<std::pair<int, int> >& pairs,
                                          int v_cnt, unsigned int e_cnt, long long tri_cnt) const;
    double GraphZero_estimate_schedule_restrict(const std::vector<int>& order,
                                                const std::vector<std::pair<int, int> >& pairs, int v_cnt,
                                                unsigned int e_cnt) const;
    double Naive_estimate_schedule_restrict(const std::vector<int>& order,
                                            const std::vector<std::pair<int, int> >& pairs, int v_cnt,
                                            unsigned int e_cnt) const;
    int get_vec_optimize_num(const std::vector<int>& vec) const;
    void remove_invalid_permutation(std::vector<std::vector<int> >& candidate_permutations) const;

    // Flat int64 tables in the layout of gpm_schedule_build (include/gpm.h).
    std::vector<int64_t> pack() const;

    std::vector<std::vector<std::vector<int> > > in_exclusion_optimize_group;
    std::vector<int> in_exclusion_optimize_val;
    std::vector<std::pair<int, int> > restrict_pair;

private:
    Schedule() = default;  // for the candidate scan
    int size = 0;
    std::vector<int> adj_mat;
    std::vector<int> father_prefix_id, last, next, loop_set_prefix_id;
    std::vector<std::vector<int> > prefix;  // member list of each prefix id
    std::vector<int> restrict_last, restrict_next, restrict_index;
    int total_prefix_num = 0;
    int total_restrict_num = 0;
    int in_exclusion_optimize_num = 0;
    long long in_exclusion_optimize_redundancy = 1;

    void init_tables();
    bool order_is_connected() const;
    void build_loop_invariant();
    int find_father_prefix(int data_size, const int* data);
    void init_in_exclusion_optimize();
    void set_in_exclusion_optimize_redundancy();
};

// Counts embeddings of `schedule` on the complete graph K_m with the same
// nested-loop semantics as Graph::pattern_matching.  Schedule construction
// uses it, as the reference does (src/schedule.cpp:1433-1456, 1746-1764),
// to validate restriction sets on K_{n+1} and to calibrate the
// inclusion–exclusion redundancy on K_n; it accepts only complete graphs.
long long complete_graph_count(const Schedule& schedule, int m);
