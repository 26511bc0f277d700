// Internal declarations shared by the host and device translation units.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <string>
#include <vector>

#include "gpm.h"

namespace gpm {

// thread-local last-error message (gpm_last_error)
void set_error(const char* fmt, ...);
void clear_error();

// Process-wide engine knobs (gpm_set_option).
struct Options {
    int64_t warps_per_block = 8;
    int64_t blocks_per_sm = 2;
    int64_t chunk = 8;          // first-level tasks per queue grab
    int64_t count_bytes = 0;    // 1: count algorithmic bytes
    int64_t timeout_ms = 2000;  // bounded device waits
    int64_t stage_max = 1024;   // largest fixed set staged in shared memory (ints)
    int64_t stage_tma = 1;      // 1: stage fixed sets with bulk copies (cp.async.bulk) instead of loads
    int64_t schedule_gpu = 1;   // 1: Schedule scores its candidates on the GPU when one is present
    int64_t leaf_batch = 0;     // 1: batched deepest level where the plan allows
    int64_t pair_leaf = 1;      // 1: pair sums over the last two levels where the plan allows
    int64_t dense_slots = 64;   // dense counter arrays for pair sums too big for a table (0 = none)
    int64_t pair_max_ops = 0;   // longest pair sum one warp takes on (0: no cap)
    int64_t pair_log2 = 0;      // log2 entries of each warp's pair-sum table (0: 17, less when memory is short)
    int64_t min_blocks = 1;     // 3: the kernel variant built for three 8-warp blocks per SM
    int64_t bitmap_min = 4096;  // fixed leaf sets this large are tested through a bitmap; 0 = never
    int64_t split = 64;         // loops this long (depth >= 2) are shared with idle warps; 0 = off
    int64_t stripes = 1;        // a launch covers chunks q*stripes + stripe only
    int64_t stripe = 0;
    int64_t raw_sums = 0;       // 1: return undivided 128-bit sums
    int64_t merge_vec = 1;      // 1: merges read 128-bit windows of the longer list
    int64_t pool = 1;           // 1: graph arrays and construction temporaries from a retained stream-ordered pool
    int64_t merge_alpha4[3] = {4, 4, 4};  // merge-vs-search weight x4 per length bucket
};
Options& options();

// Compiled schedule as the device kernels read it.
constexpr int kMaxN = 8;
constexpr int kMaxPrefix = 28;
constexpr int kMaxBlocks = 63;   // distinct inclusion–exclusion blocks (k <= 6)
constexpr int kMaxGroups = 256;
constexpr int kMaxGroupEntries = 1024;

struct DevPlan {
    int n;        // pattern vertices
    int k;        // inclusion–exclusion tail length (0: none)
    int T;        // depth of the tail (k ? n - k : n - 1)
    int L;        // deepest loop level (T - 1)
    int nprefix;
    int nslots;   // scratch slots: materialised prefixes + 2 temporaries
    int count_only;  // prefix built at level L only to be counted, or -1
    int nblocks;
    int ngroups;
    int label_sensitive;  // 1: the count depends on vertex labels; run on the caller's ids
    // Batched evaluation of the deepest loop level L (all candidates of a
    // level at once, one flat lane-balanced scan over their neighbour lists):
    //   kLeafGeneric  candidate by candidate (build_chain + tail)
    //   kLeafCount    no tail: count N(v) elements below the bound, outside
    //                 the chosen vertices and (leaf_fa >= 0) inside set leaf_fa
    //   kLeafIep2     two-loop inclusion–exclusion tail; sets a/b are
    //                 fixed (built before L), N(v), or father ∩ N(v)
    int leaf_kind;
    int leaf_fa, leaf_fb;        // probe prefix of set a / b (-1: none)
    int leaf_sa, leaf_sb;        // prefix ids of the tail's loop sets (kLeafIep2)
    int leaf_ka, leaf_kb;        // 0 fixed, 1 N(v), 2 father ∩ N(v)
    int leaf_cab, leaf_cx;       // group coefficients of |a|*|b| and |a ∩ b|
    // Pair sum over the last two loops (kLeafCount plans whose counted set is
    // N(v_{L-1}) ∩ N(v_L), whose level-L candidates and bound do not depend
    // on v_{L-1}, and whose tail bound is fixed before L-1): the count over
    // candidate pairs equals sum_x a_x * b_x - c_x, where a_x / b_x count the
    // level L-1 / L candidates adjacent to x and c_x the candidates of both.
    int pair_ok;
    int pair_pad_;
    long long redundancy;
    int loop_set[kMaxN];
    unsigned rmask[kMaxN];         // depth d stays below min(chosen[j]) for bits j
    int father[kMaxPrefix];
    int slot[kMaxPrefix];          // scratch slot of a prefix, -1 for N(v) aliases
    int chain_begin[kMaxN + 1];    // prefixes built at depth d:
    int chain_list[kMaxPrefix];    //   chain_list[chain_begin[d] .. chain_begin[d+1])
    unsigned block_mask[kMaxBlocks];   // tail positions (bit i = depth T+i) of block b
    int group_begin[kMaxGroups + 1];
    int group_coef[kMaxGroups];
    unsigned char group_block[kMaxGroupEntries];
};

constexpr int kLeafGeneric = 0, kLeafCount = 1, kLeafIep2 = 2;

// Scores schedule candidates on the GPU (schedule_gpu.cu): candidate c is
// the pattern in loop order cand_order[c] (mats holds n*n ints per order)
// with npairs[c] sorted restriction pairs (28 slots of two ints each in
// pairs); perf is the performance model (1..3).  GPM_ERR_NO_DEVICE without a
// GPU.  The values equal the host models' bit for bit.
int score_candidates_gpu(int n, int perf, int pattern_max_degree, const std::vector<int>& mats,
                         const std::vector<int>& cand_order, const std::vector<int>& npairs,
                         const std::vector<int>& pairs, int v_cnt, unsigned int e_cnt, long long tri_cnt,
                         std::vector<double>& vals);

// Decodes gpm_schedule_build tables into a DevPlan (host).
int compile_plan(const int64_t* t, int32_t n_words, DevPlan* out);

// Host model of the device enumeration for a plan on a small CSR: the raw
// signed sum before the division by the redundancy.
__int128 plan_probe_count(const DevPlan& p, int v_cnt, const std::vector<uint32_t>& rowptr,
                          const std::vector<int32_t>& col);

// 1 when the plan's count changes with the vertex labelling (see
// compile_plan), 0 otherwise.
int plan_label_sensitive(const DevPlan& p);

}  // namespace gpm

struct gpm_plan {
    gpm::DevPlan host;
    gpm::DevPlan* dev = nullptr;
    int device = 0;
};

struct gpm_graph {
    int32_t v_cnt = 0;
    uint64_t e_cnt = 0;
    int32_t max_degree = 0;
    int32_t max_isect = 0;
    uint32_t* rowptr = nullptr;  // device, relabelled by degree when relabelled
    int32_t* col = nullptr;      // device
    uint32_t* orig_rowptr = nullptr;  // device, the caller's ids (== rowptr when not relabelled)
    int32_t* orig_col = nullptr;
    int device = 0;
    bool relabelled = false;
    bool pooled = false;     // the arrays come from the device's stream-ordered pool
    void* stream = nullptr;  // the stream their pooled frees are ordered on
};
