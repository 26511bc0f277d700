// GB300 (sm_103a) kernels and the device half of the C ABI.
//
// The hot path is the schedule-driven nested-loop enumeration of
// Graph::pattern_matching / pattern_matching_aggressive_func
// (reference src/graph.cpp:199-398), re-planned for the GPU:
//   * persistent warps pull first-level edges (v0, v1) — or root vertices
//     when the tail starts at depth 1 — from per-(pattern, graph) atomic
//     work queues; a chunk of consecutive edges shares v0;
//   * every prefix set (VertexSet::build_vertex_set, src/vertex_set.cpp:158)
//     is built by a warp-cooperative intersection: lanes take 32 elements of
//     the smaller sorted list, binary-search the larger one from a moving
//     lower bound, and compact hits with __ballot_sync/__popc;
//   * the last loop's set is never written out: its size below the
//     restriction bound and minus the chosen vertices is counted during the
//     intersection (src/graph.cpp:346-364 fused with :383-390);
//   * the inclusion–exclusion tail (src/graph.cpp:306-344) evaluates each
//     distinct block once and combines groups in 128-bit integers;
//   * per-warp sums are 128-bit and reach the per-pair result through two
//     64-bit atomics with carry, so counts above 2^64 stay exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include <cub/cub.cuh>

#include "gpm_internal.h"

namespace gpm {

#define GPM_CK(call)                                                                               \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return e_ == cudaErrorMemoryAllocation ? GPM_ERR_OOM : GPM_ERR_CUDA;                  \
        }                                                                                          \
    } while (0)

constexpr unsigned kFull = 0xffffffffu;

// Internal-check record: the first kernel that detects an impossible state
// (a merge window that does not advance, an id outside the graph) writes a
// code and a few values here and skips the work; the host reports it.
// [0] code, [1..7] values.
constexpr int kErrMergeStall = 1, kErrBadVertex = 2;
__device__ unsigned long long g_check[8];

__device__ __noinline__ void record_check(int code, long long a, long long b, long long c, long long d, long long e,
                                          long long f) {
    if (atomicCAS(&g_check[0], 0ull, (unsigned long long)code) == 0ull) {
        g_check[1] = (unsigned long long)a;
        g_check[2] = (unsigned long long)b;
        g_check[3] = (unsigned long long)c;
        g_check[4] = (unsigned long long)d;
        g_check[5] = (unsigned long long)e;
        g_check[6] = (unsigned long long)f;
        __threadfence();
    }
}

// ---------------------------------------------------------------------------
// device building blocks

struct GraphView {
    const unsigned* __restrict__ rowptr;
    const int* __restrict__ col;
    int v_cnt;
    int pad_;
    unsigned long long e_cnt;
};

struct PairDesc {
    GraphView g;
    const DevPlan* plan;
    unsigned long long ntasks;  // v_cnt when the tail starts at depth 1, else e_cnt
    int cap;                    // scratch ints per slot for this graph
    int pad_;
};

struct WarpState {
    int chosen[kMaxN];
    int idx[kMaxN];
    int end[kMaxN];
    int len[kMaxPrefix];
    const int* ptr[kMaxPrefix];
    const int* lp[kMaxN];
    int blockval[kMaxBlocks];
    int leafcnt[3][32];  // per-candidate counters of a leaf batch
    unsigned epoch;      // tag of the live entries of this warp's pair-sum table
    int dslot[kMaxN];    // donation record the loop of depth d draws from (-1: none)
    unsigned dgen[kMaxN];
    int downer[kMaxN];   // 1: this warp published that record
};

// Work donation (hub splitting).  A warp whose loop at depth d >= 2 has at
// least `split` candidates publishes the loop as a record: the pair, d and
// chosen[0, d).  From then on the owner and any warp that has finished its
// own queues take slices [next, next + s) of the loop by compare-and-swap on
// the record's word; a helper rebuilds the prefix sets of chosen[0, d) and
// adds what it counts to the pair's sum.  Nothing waits on a record: a warp
// that finds no free slot runs its loop alone, a claim either succeeds or
// sees the loop exhausted, and only the owner frees a slot, after the last
// slice has been taken (helpers keep their own copies of what they need).
constexpr int kDonSlots = 1024;
constexpr int kErrDonation = 4;

struct Donation {
    unsigned long long word;  // generation (16 bits) | end (24) | next (24)
    int pair;
    int depth;
    int chosen[kMaxN];
    int pad_[4];
};
static_assert(sizeof(Donation) == 64, "one record per 64 bytes");

struct DonationArea {
    Donation rec[kDonSlots];
    unsigned busy[kDonSlots];  // 1 while a record's owner holds the slot
    unsigned finished;         // warps done with their own queues
    unsigned pad_[3];
};

__device__ __forceinline__ unsigned long long don_pack(unsigned gen, unsigned end, unsigned next) {
    return ((unsigned long long)(gen & 0xffffu) << 48) | ((unsigned long long)(end & 0xffffffu) << 24) |
           (unsigned long long)(next & 0xffffffu);
}

// Takes the next slice of record r (generation gen); lo == hi when the loop
// is exhausted or the slot holds another generation.  Lock-free: a failed
// compare-and-swap means another warp took a slice, so the retries are
// bounded by the loop length (< 2^24).
__device__ void don_claim(Donation* r, unsigned gen, int& lo, int& hi) {
    lo = hi = 0;
    unsigned long long w = *(volatile unsigned long long*)&r->word;
    for (int tries = 0; tries < (1 << 25); ++tries) {
        if ((unsigned)(w >> 48) != (gen & 0xffffu)) return;
        const unsigned end = (unsigned)(w >> 24) & 0xffffffu, next = (unsigned)w & 0xffffffu;
        if (next >= end) return;
        const unsigned take = min(64u, max(1u, (end - next) >> 5));
        const unsigned long long got = atomicCAS(&r->word, w, don_pack(gen, end, next + take));
        if (got == w) {
            lo = (int)next;
            hi = (int)(next + take);
            return;
        }
        w = got;
    }
    record_check(kErrDonation, gen, (long long)w, 0, 0, 0, 0);
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// first index i in a[0, n) with a[i] >= x (all lanes search the same key)
__device__ __forceinline__ int lower_bound_u(const int* a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Merge variant: both lists advance through 32-wide coalesced windows; each
// lane locates its A element in the B window with a 5-step shuffle search.
// Elements of A no larger than the last B of the window are resolved and
// consumed, likewise for B, so each step consumes a full window of at least
// one list.  Found elements are compacted in order (kStore) or counted minus
// the chosen vertices.
template <bool kStore>
__device__ int warp_merge(const int* A, int na, const int* B, int nb, int* out, const int* chosen, int nch,
                          int lane) {
    int i = 0, j = 0, acc = 0;
    while (i < na && j < nb) {
        const int a = (i + lane < na) ? A[i + lane] : INT_MAX;
        const int b = (j + lane < nb) ? B[j + lane] : INT_MAX;
        int pos = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int bv = __shfl_sync(kFull, b, pos + step - 1);
            if (bv < a) pos += step;
        }
        // every lane must execute the shuffle (no short-circuit around it)
        const int bp = __shfl_sync(kFull, b, pos);
        bool found = (a != INT_MAX) && (bp == a);
        if (!kStore && found)
            for (int q = 0; q < nch; ++q)
                if (chosen[q] == a) found = false;
        const unsigned fm = __ballot_sync(kFull, found);
        if (kStore && found) out[acc + __popc(fm & lanemask_lt())] = a;
        acc += __popc(fm);
        const int amax = __shfl_sync(kFull, a, 31), bmax = __shfl_sync(kFull, b, 31);
        const int di = __popc(__ballot_sync(kFull, a <= bmax));
        const int dj = __popc(__ballot_sync(kFull, b <= amax));
        if (di == 0 && dj == 0) {
            // only possible when a window is not sorted: record and stop
            const int a0 = __shfl_sync(kFull, a, 0);
            if (lane == 0) record_check(kErrMergeStall, na, nb, i, j, a0, bmax);
            break;
        }
        i += di;
        j += dj;
    }
    if (kStore) __syncwarp();
    return acc;
}

// Merge when both lists are of similar length: a binary-search round costs
// about log2(nb) dependent loads for 32 elements of the short list, a merge
// step one coalesced load per list for at least 32 elements.
// alpha4 = 4 x the weight of a binary-search round, per bucket of the longer
// list's length (< 256, < 8192, larger); the autotuner sets them.
__constant__ int c_merge_alpha4[3] = {4, 4, 4};

__device__ __forceinline__ bool prefer_merge(int na, int nb) {
    const int lg = 32 - __clz(nb | 1);
    const int a4 = c_merge_alpha4[nb < 256 ? 0 : (nb < 8192 ? 1 : 2)];
    return (long long)na * lg * a4 >= 4ll * (long long)(na + nb);
}

// A ∩ B written sorted to out; returns its size.
__device__ int isect_store(const int* A, int na, const int* B, int nb, int* out, int lane) {
    if (na > nb) {
        const int* t = A; A = B; B = t;
        int u = na; na = nb; nb = u;
    }
    if (prefer_merge(na, nb)) return warp_merge<true>(A, na, B, nb, out, nullptr, 0, lane);
    int written = 0, lo = 0;
    for (int base = 0; base < na; base += 32) {
        const int i = base + lane;
        const bool valid = i < na;
        const int x = valid ? A[i] : INT_MAX;
        int l = lo, h = nb;
        while (l < h) {
            int m = (l + h) >> 1;
            if (B[m] < x) l = m + 1;
            else h = m;
        }
        const bool found = valid && l < nb && B[l] == x;
        const unsigned mask = __ballot_sync(kFull, found);
        if (found) out[written + __popc(mask & lanemask_lt())] = x;
        written += __popc(mask);
        lo = __shfl_sync(kFull, l, 31);
    }
    __syncwarp();
    return written;
}

// |A ∩ B ∩ [0, bound) \ chosen[0, nch)|
__device__ int isect_count(const int* A, int na, const int* B, int nb, int bound, const int* chosen, int nch,
                           int lane) {
    na = lower_bound_u(A, na, bound);
    nb = lower_bound_u(B, nb, bound);
    if (na > nb) {
        const int* t = A; A = B; B = t;
        int u = na; na = nb; nb = u;
    }
    if (prefer_merge(na, nb)) return warp_merge<false>(A, na, B, nb, nullptr, chosen, nch, lane);
    int cnt = 0, lo = 0;
    for (int base = 0; base < na; base += 32) {
        const int i = base + lane;
        const bool valid = i < na;
        const int x = valid ? A[i] : INT_MAX;
        int l = lo, h = nb;
        while (l < h) {
            int m = (l + h) >> 1;
            if (B[m] < x) l = m + 1;
            else h = m;
        }
        bool found = valid && l < nb && B[l] == x;
        if (found)
            for (int j = 0; j < nch; ++j)
                if (chosen[j] == x) found = false;
        cnt += __popc(__ballot_sync(kFull, found));
        lo = __shfl_sync(kFull, l, 31);
    }
    return cnt;
}

// |S[0, len) \ chosen[0, nch)|  (VertexSet::unorderd_subtraction_size,
// src/vertex_set.cpp:196-209)
__device__ __forceinline__ int count_outside(const int* S, int len, const int* chosen, int nch, int lane) {
    bool in = false;
    if (lane < nch) {
        const int c = chosen[lane];
        const int p = lower_bound_u(S, len, c);
        in = p < len && S[p] == c;
    }
    return len - __popc(__ballot_sync(kFull, in));
}

__device__ __forceinline__ void add128(unsigned long long* o, __int128 v) {
    const unsigned long long lo = (unsigned long long)v;
    const unsigned long long hi = (unsigned long long)(v >> 64);
    const unsigned long long old = atomicAdd(o, lo);
    const unsigned long long carry = (old + lo < old) ? 1ull : 0ull;
    if (hi + carry) atomicAdd(o + 1, hi + carry);
}

// Pair-sum table entries: epoch (16 bits) | vertex (24 bits) | count (24 bits).
// A slot whose epoch differs from the warp's current one is empty.
__device__ __forceinline__ unsigned long long pair_word(unsigned epoch, int x, unsigned cnt) {
    return ((unsigned long long)(epoch & 0xffffu) << 48) | ((unsigned long long)(x & 0xffffff) << 24) | cnt;
}

__device__ __forceinline__ unsigned pair_slot(int x, unsigned mask) { return ((unsigned)x * 2654435761u) >> 7 & mask; }

// adds one to x's count; false when the table is full (never at load <= 1/2)
__device__ bool pair_add(unsigned long long* T, unsigned mask, unsigned epoch, int x) {
    unsigned slot = pair_slot(x, mask);
    for (unsigned probes = 0; probes <= mask; ++probes) {
        unsigned long long old = T[slot];
        for (;;) {
            const bool live = (unsigned)(old >> 48) == (epoch & 0xffffu);
            if (live && (int)((old >> 24) & 0xffffff) == x) {
                const unsigned long long got = atomicCAS(&T[slot], old, old + 1);
                if (got == old) return true;
                old = got;
                continue;
            }
            if (!live) {
                const unsigned long long got = atomicCAS(&T[slot], old, pair_word(epoch, x, 1));
                if (got == old) return true;
                old = got;
                continue;
            }
            break;  // live entry of another vertex: next slot
        }
        slot = (slot + 1) & mask;
    }
    return false;
}

__device__ unsigned pair_get(const unsigned long long* T, unsigned mask, unsigned epoch, int x) {
    unsigned slot = pair_slot(x, mask);
    for (unsigned probes = 0; probes <= mask; ++probes) {
        const unsigned long long w = T[slot];
        if ((unsigned)(w >> 48) != (epoch & 0xffffu)) return 0;
        if ((int)((w >> 24) & 0xffffff) == x) return (unsigned)(w & 0xffffff);
        slot = (slot + 1) & mask;
    }
    return 0;
}

// x in sorted a[0, n) (per-lane search)
__device__ __forceinline__ bool contains(const int* a, int n, int x) {
    const int p = lower_bound_u(a, n, x);
    return p < n && a[p] == x;
}

template <bool kBytes>
struct WarpCtx {
    WarpState* s;
    const DevPlan* __restrict__ P;
    GraphView g;
    int* scratch;
    int cap;
    int lane;
    int leaf_on;
    int* stage;      // 2 * stage_cap ints of this warp's shared memory
    int stage_cap;
    int pair_on;
    unsigned long long* ptab;  // this warp's pair-sum table (pmask + 1 words)
    unsigned pmask;
    DonationArea* don;         // null: no donation
    int split_min;             // smallest loop that is donated
    int pair_idx;              // pair whose work is running
    long long gw;              // global warp index
    unsigned long long bytes;

    // copies a fixed set into shared-memory region r when it fits
    __device__ const int* stage_set(const int* p, int n, int r) {
        if (n > stage_cap || n <= 0) return p;
        int* dst = stage + r * stage_cap;
        for (int i = lane; i < n; i += 32) dst[i] = p[i];
        __syncwarp();
        return dst;
    }

    // Exclusive scan of len over the warp; returns the total.
    __device__ __forceinline__ int warp_scan(int len, int& pre) const {
        int incl = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        pre = incl - len;
        return __shfl_sync(kFull, incl, 31);
    }

    // owner lane of flat element e: the largest lane c with pre_c <= e
    __device__ __forceinline__ int owner(int pre, int e) const {
        int c = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int q = c + step;
            const int pq = __shfl_sync(kFull, pre, q & 31);
            if (q < 32 && pq <= e) c = q;
        }
        return c;
    }

    __device__ __forceinline__ bool chosen_before(int x, int L) const {
        bool hit = false;
        for (int q = 0; q < L; ++q) hit |= s->chosen[q] == x;
        return hit;
    }

    // Sum over (v, w), v a level L-1 candidate, w a level L candidate, v != w,
    // of |N(v) ∩ N(w) ∩ [0, bound) \ chosen|, as sum_x a_x b_x - c_x (the
    // plan's pair_ok shape).  Level L-1's loop list is set.  Returns false
    // (and does nothing) when B's neighbour lists would fill the table more
    // than half: the caller then runs the level normally.
    __device__ bool pair_level(__int128& out) {
        const int L1 = P->L - 1;
        const int T = P->T;
        const int* candA = s->lp[L1];
        const int na = s->end[L1];
        const int sb = P->loop_set[P->L];
        const int* candB = s->ptr[sb];
        const int nb = lower_bound_u(candB, s->len[sb], bound_of(P->L));
        const int bnd = bound_of(T);
        // size of B's neighbour lists below the bound
        long long mb = 0;
        for (int base = 0; base < nb; base += 32) {
            const int j = base + lane;
            int len = 0;
            if (j < nb) {
                const int w = candB[j];
                if (!chosen_before(w, L1)) {
                    const unsigned st = g.rowptr[w];
                    len = lower_bound_u(g.col + st, (int)(g.rowptr[w + 1] - st), bnd);
                }
            }
            int pre;
            mb += warp_scan(len, pre);
        }
        if (mb * 2 > (long long)pmask + 1) return false;
        if (lane == 0) {
            s->epoch = (s->epoch + 1) & 0xffffu;
            if (s->epoch == 0) s->epoch = 1;
        }
        __syncwarp();
        const unsigned ep = s->epoch;
        if (ep == 1) {  // fresh cycle of tags: clear the table
            for (unsigned i = lane; i <= pmask; i += 32) ptab[i] = 0ull;
            __syncwarp();
        }
        long long sum = 0;
        // phase 1 (B -> counts) and phase 2 (A -> sum of counts)
        for (int phase = 0; phase < 2; ++phase) {
            const int* cand = phase == 0 ? candB : candA;
            const int nc = phase == 0 ? nb : na;
            for (int base = 0; base < nc; base += 32) {
                const int j = base + lane;
                unsigned st = 0;
                int len = 0;
                if (j < nc) {
                    const int v = cand[j];
                    if (!chosen_before(v, L1)) {
                        st = g.rowptr[v];
                        len = lower_bound_u(g.col + st, (int)(g.rowptr[v + 1] - st), bnd);
                        if (kBytes) bytes += 4ull * (unsigned long long)len + 8;
                    }
                }
                int pre;
                const int M = warp_scan(len, pre);
                for (int eb = 0; eb < M; eb += 32) {
                    const int e = eb + lane;
                    const int c = owner(pre, e);
                    const unsigned stc = __shfl_sync(kFull, st, c);
                    const int prc = __shfl_sync(kFull, pre, c);
                    if (e < M) {
                        const int x = g.col[stc + (e - prc)];
                        if (!chosen_before(x, L1)) {
                            if (phase == 0) {
                                if (!pair_add(ptab, pmask, ep, x)) record_check(3, x, mb, pmask, 0, 0, 0);
                            } else {
                                sum += pair_get(ptab, pmask, ep, x);
                            }
                        }
                    }
                }
                __syncwarp();
            }
        }
        // c term: v in both candidate lists pairs with itself
        for (int base = 0; base < na; base += 32) {
            const int j = base + lane;
            if (j < na) {
                const int v = candA[j];
                if (!chosen_before(v, L1) && contains(candB, nb, v)) {
                    const unsigned st = g.rowptr[v];
                    const int* nv = g.col + st;
                    const int len = lower_bound_u(nv, (int)(g.rowptr[v + 1] - st), bnd);
                    int in = 0;
                    for (int q = 0; q < L1; ++q) in += contains(nv, len, s->chosen[q]) ? 1 : 0;
                    sum -= (long long)(len - in);
                }
            }
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
        out = lane == 0 ? (__int128)sum : (__int128)0;
        return true;
    }

    // All candidates of level L at once (the plan's leaf_kind says how the
    // tail reads N(v)); chosen[0, L) and the level's loop list are set.
    __device__ __int128 leaf_batch() {
        const int L = P->L, T = P->T;
        const int* cand = s->lp[L];
        const int ncand = s->end[L];
        long long total = 0;
        if (P->leaf_kind == kLeafCount) {
            // bound of the last loop: restrictions on depths < L are fixed
            const unsigned m = P->rmask[T];
            int bfix = g.v_cnt;
            for (int j = 0; j < L; ++j)
                if (m >> j & 1) bfix = min(bfix, s->chosen[j]);
            const bool by_v = (m >> L) & 1;
            const int* F = nullptr;
            int nf = 0, lim = bfix;
            if (P->leaf_fa >= 0) {
                nf = lower_bound_u(s->ptr[P->leaf_fa], s->len[P->leaf_fa], bfix);
                if (nf == 0) return 0;
                F = stage_set(s->ptr[P->leaf_fa], nf, 0);
                lim = min(bfix, F[nf - 1] + 1);
            }
            for (int base = 0; base < ncand; base += 32) {
                const int j = base + lane;
                bool ok = j < ncand;
                const int v = ok ? cand[j] : 0;
                if (ok) ok = !chosen_before(v, L);
                unsigned st = 0;
                int len = 0;
                if (ok) {
                    st = g.rowptr[v];
                    const int dv = (int)(g.rowptr[v + 1] - st);
                    len = lower_bound_u(g.col + st, dv, by_v ? min(lim, v) : lim);
                    if (kBytes) bytes += 4ull * (unsigned long long)(s->len[P->leaf_fa >= 0 ? P->leaf_fa : 0] * (P->leaf_fa >= 0) + dv) + 8;
                }
                int pre;
                const int M = warp_scan(len, pre);
                for (int eb = 0; eb < M; eb += 32) {
                    const int e = eb + lane;
                    const int c = owner(pre, e);
                    const unsigned stc = __shfl_sync(kFull, st, c);
                    const int prc = __shfl_sync(kFull, pre, c);
                    bool hit = false;
                    if (e < M) {
                        const int x = g.col[stc + (e - prc)];
                        hit = !chosen_before(x, L);
                        if (hit && F) hit = contains(F, nf, x);
                    }
                    total += __popc(__ballot_sync(kFull, hit));
                }
            }
            return lane == 0 ? (__int128)total : (__int128)0;
        }
        // ---- two-loop inclusion–exclusion tail ----
        const int sa = P->leaf_sa, sb = P->leaf_sb, ka = P->leaf_ka, kb = P->leaf_kb;
        const bool same = sa == sb, both_fixed = ka == 0 && kb == 0;
        const int* Pa = nullptr;
        const int* Pb = nullptr;
        int na = 0, nb = 0;
        if (P->leaf_fa >= 0) {
            na = s->len[P->leaf_fa];
            Pa = stage_set(s->ptr[P->leaf_fa], na, 0);
        }
        if (P->leaf_fb >= 0) {
            nb = s->len[P->leaf_fb];
            Pb = (P->leaf_fb == P->leaf_fa) ? Pa : stage_set(s->ptr[P->leaf_fb], nb, 1);
        }
        const int fixA = ka == 0 ? count_outside(s->ptr[sa], s->len[sa], s->chosen, L, lane) : 0;
        const int fixB = kb == 0 ? count_outside(s->ptr[sb], s->len[sb], s->chosen, L, lane) : 0;
        const int fixX = (both_fixed && !same)
                             ? isect_count(s->ptr[sa], s->len[sa], s->ptr[sb], s->len[sb], INT_MAX, s->chosen, L, lane)
                             : 0;
        const long long cab = P->leaf_cab, cx = P->leaf_cx;
        for (int base = 0; base < ncand; base += 32) {
            const int j = base + lane;
            bool ok = j < ncand;
            const int v = ok ? cand[j] : 0;
            if (ok) ok = !chosen_before(v, L);
            unsigned st = 0;
            int len = 0;
            bool inA = false, inB = false;
            if (ok) {
                if (ka == 0) inA = contains(Pa, na, v);
                if (kb == 0) inB = contains(Pb, nb, v);
                if (!both_fixed) {
                    st = g.rowptr[v];
                    len = (int)(g.rowptr[v + 1] - st);
                }
            }
            s->leafcnt[0][lane] = 0;
            s->leafcnt[1][lane] = 0;
            s->leafcnt[2][lane] = 0;
            __syncwarp();
            int pre;
            const int M = warp_scan(len, pre);
            for (int eb = 0; eb < M; eb += 32) {
                const int e = eb + lane;
                const int c = owner(pre, e);
                const unsigned stc = __shfl_sync(kFull, st, c);
                const int prc = __shfl_sync(kFull, pre, c);
                bool ma = false, mb = false;
                if (e < M) {
                    const int x = g.col[stc + (e - prc)];
                    if (!chosen_before(x, L)) {
                        ma = ka == 1 ? true : contains(Pa, na, x);
                        mb = kb == 1 ? true : contains(Pb, nb, x);
                    }
                }
                const unsigned grp = __match_any_sync(kFull, e < M ? c : 32 + lane);
                const unsigned ba = __ballot_sync(kFull, ma), bb = __ballot_sync(kFull, mb),
                               bx = __ballot_sync(kFull, ma && mb);
                if (e < M && lane == __ffs(grp) - 1) {
                    s->leafcnt[0][c] += __popc(ba & grp);
                    s->leafcnt[1][c] += __popc(bb & grp);
                    s->leafcnt[2][c] += __popc(bx & grp);
                }
                __syncwarp();
            }
            if (ok) {
                const long long A = ka == 0 ? (long long)(fixA - (inA ? 1 : 0)) : s->leafcnt[0][lane];
                const long long B = kb == 0 ? (long long)(fixB - (inB ? 1 : 0)) : s->leafcnt[1][lane];
                const long long X = same ? A : (both_fixed ? (long long)(fixX - (inA && inB ? 1 : 0)) : s->leafcnt[2][lane]);
                total += cab * A * B + cx * X;
                if (kBytes) bytes += 4ull * (unsigned long long)(len + (ka == 2 ? na : 0) + (kb == 2 ? nb : 0) + A + B) + 8;
            }
            __syncwarp();
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) total += __shfl_xor_sync(kFull, total, o);
        return lane == 0 ? (__int128)total : (__int128)0;
    }

    __device__ __forceinline__ void nbr(int v, const int*& p, int& d) const {
        const unsigned a = g.rowptr[v], b = g.rowptr[v + 1];
        p = g.col + a;
        d = (int)(b - a);
    }

    __device__ __forceinline__ int bound_of(int d) const {
        unsigned m = P->rmask[d];
        int b = g.v_cnt;
        while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            b = min(b, s->chosen[j]);
        }
        return b;
    }

    __device__ __forceinline__ bool in_chosen(int v, int d) const {
        bool hit = false;
        for (int j = 0; j < d; ++j) hit |= s->chosen[j] == v;
        return hit;
    }

    __device__ __forceinline__ void set_chosen(int d, int v) {
        if (lane == 0) s->chosen[d] = v;
        __syncwarp();
    }

    // Builds the prefix sets whose last member is depth d for candidate v.
    __device__ bool build_chain(int d, const int* nv, int dv) {
        const int b = P->chain_begin[d], e = P->chain_begin[d + 1];
        for (int c = b; c < e; ++c) {
            const int pid = P->chain_list[c];
            const int f = P->father[pid];
            const int* ptr;
            int len;
            if (f < 0) {
                ptr = nv;
                len = dv;
            } else {
                int* dst = scratch + (size_t)P->slot[pid] * cap;
                const int lf = s->len[f];
                len = isect_store(s->ptr[f], lf, nv, dv, dst, lane);
                ptr = dst;
                if (kBytes) bytes += 4ull * (unsigned long long)(lf + dv);
            }
            if (lane == 0) {
                s->ptr[pid] = ptr;
                s->len[pid] = len;
            }
            __syncwarp();
            if (len == 0) return false;
        }
        return true;
    }

    // inclusion–exclusion tail at depth T (src/graph.cpp:306-344)
    __device__ __int128 iep_tail() {
        const int T = P->T, k = P->k;
        for (int i = 0; i < k; ++i) {
            const int sid = P->loop_set[T + i];
            const int v = count_outside(s->ptr[sid], s->len[sid], s->chosen, T, lane);
            if (v == 0) return 0;  // every group holds a block inside S_i
            if (lane == 0) s->blockval[i] = v;
        }
        const int tmp0 = P->nslots - 2;
        for (int b = k; b < P->nblocks; ++b) {
            unsigned m = P->block_mask[b];
            int j = __ffs(m) - 1;
            m &= m - 1;
            const int* A = s->ptr[P->loop_set[T + j]];
            int na = s->len[P->loop_set[T + j]];
            int flip = 0;
            while (__popc(m) > 1 && na > 0) {
                j = __ffs(m) - 1;
                m &= m - 1;
                const int sid = P->loop_set[T + j];
                int* dst = scratch + (size_t)(tmp0 + flip) * cap;
                if (kBytes) bytes += 4ull * (unsigned long long)(na + s->len[sid]);
                na = isect_store(A, na, s->ptr[sid], s->len[sid], dst, lane);
                A = dst;
                flip ^= 1;
            }
            int val = 0;
            if (na > 0) {
                j = __ffs(m) - 1;
                const int sid = P->loop_set[T + j];
                if (kBytes) bytes += 4ull * (unsigned long long)(na + s->len[sid]);
                val = isect_count(A, na, s->ptr[sid], s->len[sid], INT_MAX, s->chosen, T, lane);
            }
            if (lane == 0) s->blockval[b] = val;
        }
        __syncwarp();
        __int128 total = 0;
        if (lane == 0) {
            for (int g2 = 0; g2 < P->ngroups; ++g2) {
                __int128 v = P->group_coef[g2];
                for (int q = P->group_begin[g2]; q < P->group_begin[g2 + 1]; ++q) {
                    v *= (__int128)s->blockval[P->group_block[q]];
                    if (v == 0) break;
                }
                total += v;
            }
        }
        return total;
    }

    // the reference's work at depth T once chosen[0, T) and all sets exist
    __device__ __int128 tail_at_T() {
        const int T = P->T;
        const int sid = P->loop_set[T];
        const int len = s->len[sid];
        if (len <= 0) return 0;
        if (P->k) return iep_tail();
        const int* S = s->ptr[sid];
        const int lb = lower_bound_u(S, len, bound_of(T));
        return (__int128)count_outside(S, lb, s->chosen, T, lane);
    }

    // candidate v at the deepest loop level L
    __device__ __int128 tail_with_candidate(int v, const int* nv, int dv) {
        const int L = P->L;
        if (P->count_only >= 0) {
            set_chosen(L, v);
            const int f = P->father[P->count_only];
            if (kBytes) bytes += 4ull * (unsigned long long)(s->len[f] + dv);
            return (__int128)isect_count(s->ptr[f], s->len[f], nv, dv, bound_of(P->T), s->chosen, P->T, lane);
        }
        if (!build_chain(L, nv, dv)) return 0;
        set_chosen(L, v);
        return tail_at_T();
    }

    __device__ void start_level(int d) {
        const int sid = P->loop_set[d];
        const int* S = s->ptr[sid];
        const int e = lower_bound_u(S, s->len[sid], bound_of(d));
        if (lane == 0) {
            s->lp[d] = S;
            s->idx[d] = 0;
            s->end[d] = e;
            s->dslot[d] = -1;
        }
        __syncwarp();
    }

    // Publishes the loop of depth d (just started) when it is long enough
    // and a slot is free; the owner's own range then comes from claims.
    __device__ void maybe_donate(int d) {
        if (!don || split_min <= 0) return;
        const int e = s->end[d];
        if (e < split_min || e > 0xffffff) return;
        if (lane == 0) {
            int h = -1;
            for (int probe = 0; probe < 4 && h < 0; ++probe) {
                const int c = (int)((gw * 7 + d * 131 + probe * 257) & (kDonSlots - 1));
                if (atomicCAS(&don->busy[c], 0u, 1u) == 0u) h = c;
            }
            if (h >= 0) {
                Donation* r = &don->rec[h];
                volatile Donation* vr = r;
                const unsigned gen = ((unsigned)(vr->word >> 48) + 1u) & 0xffffu;
                vr->pair = pair_idx;
                vr->depth = d;
                for (int j = 0; j < d; ++j) vr->chosen[j] = s->chosen[j];
                __threadfence();
                atomicExch(&r->word, don_pack(gen, (unsigned)e, 0u));
                s->dslot[d] = h;
                s->dgen[d] = gen;
                s->downer[d] = 1;
                s->end[d] = 0;
            }
        }
        __syncwarp();
    }

    // next slice of the donated loop at depth d into idx[d], end[d]
    __device__ bool claim_more(int d) {
        int lo = 0, hi = 0;
        if (lane == 0) {
            don_claim(&don->rec[s->dslot[d]], s->dgen[d], lo, hi);
            if (hi > lo) {
                s->idx[d] = lo;
                s->end[d] = hi;
            }
        }
        hi = __shfl_sync(kFull, hi, 0);
        lo = __shfl_sync(kFull, lo, 0);
        __syncwarp();
        return hi > lo;
    }

    // the donated loop at depth d is exhausted: its owner frees the slot
    __device__ void release(int d) {
        if (lane == 0) {
            if (s->downer[d]) {
                __threadfence();
                atomicExch(&don->busy[s->dslot[d]], 0u);
            }
            s->dslot[d] = -1;
        }
        __syncwarp();
    }

    __device__ __forceinline__ bool batch_on() const { return leaf_on && P->leaf_kind != kLeafGeneric; }
    // pair-sum table keys are 24-bit ids
    __device__ __forceinline__ bool pair_ready() const { return pair_on && P->pair_ok && g.v_cnt <= (1 << 24); }

    // Loops of depths d0..L; chosen[0, d0), their prefix sets and the loop
    // range of depth d0 are set.  Returns when depth d0's range (and, for a
    // donated loop, every slice of it) is done.
    __device__ __int128 dfs_levels(int d0) {
        const int L = P->L;
        const bool batch = batch_on();
        const bool pair = pair_ready();
        __int128 acc = 0;
        int d = d0;
        while (d >= d0) {
            const int i = s->idx[d];
            if (i >= s->end[d]) {
                if (s->dslot[d] >= 0) {
                    if (claim_more(d)) continue;
                    release(d);
                }
                --d;
                continue;
            }
            const int v = s->lp[d][i];
            __syncwarp();
            if (lane == 0) s->idx[d] = i + 1;
            __syncwarp();
            if (in_chosen(v, d)) continue;
            const int* nv;
            int dv;
            nbr(v, nv, dv);
            if (kBytes) bytes += 8;
            if (d == L) {
                acc += tail_with_candidate(v, nv, dv);
                continue;
            }
            if (!build_chain(d, nv, dv)) continue;
            set_chosen(d, v);
            ++d;
            start_level(d);
            if (batch && d == L) {
                acc += leaf_batch();
                --d;
                continue;
            }
            if (pair && d == L - 1) {
                __int128 r;
                if (pair_level(r)) {
                    acc += r;
                    --d;
                    continue;
                }
            }
            maybe_donate(d);
        }
        return acc;
    }

    // levels 2..L below a fixed (v0, v1)
    __device__ __int128 dfs_from_2() {
        const int L = P->L;
        start_level(2);
        if (batch_on() && L == 2) return leaf_batch();
        if (pair_ready() && L == 3) {
            __int128 r;
            if (pair_level(r)) return r;
        }
        maybe_donate(2);
        return dfs_levels(2);
    }

    // Takes slices of record h (generation gen) until it is exhausted;
    // false when nothing could be taken.
    __device__ bool help_one(const PairDesc* pairs, int npairs, unsigned long long* out, int h, unsigned gen) {
        Donation* r = &don->rec[h];
        int lo = 0, hi = 0, p = 0, d = 0, rend = 0;
        if (lane == 0) {
            const unsigned long long w = *(volatile unsigned long long*)&r->word;
            if ((unsigned)(w >> 48) == gen && (w & 0xffffffu) < ((w >> 24) & 0xffffffu)) {
                __threadfence();
                const volatile Donation* vr = r;
                p = vr->pair;
                d = vr->depth;
                for (int j = 0; j < kMaxN; ++j) s->chosen[j] = j < d ? vr->chosen[j] : -1;
                rend = (int)((w >> 24) & 0xffffffu);
                // the claim succeeds only while the record still holds these fields
                don_claim(r, gen, lo, hi);
            }
        }
        lo = __shfl_sync(kFull, lo, 0);
        hi = __shfl_sync(kFull, hi, 0);
        p = __shfl_sync(kFull, p, 0);
        d = __shfl_sync(kFull, d, 0);
        rend = __shfl_sync(kFull, rend, 0);
        __syncwarp();
        if (hi <= lo) return false;
        if (p < 0 || p >= npairs) {
            if (lane == 0) record_check(kErrDonation, h, p, d, lo, hi, rend);
            __syncwarp();
            return true;
        }
        const PairDesc pd = pairs[p];
        P = pd.plan;
        g = pd.g;
        cap = pd.cap;
        pair_idx = p;
        bool ok = d >= 2 && d <= P->L;
        for (int l = 0; l < d && ok; ++l) {
            const int* nv;
            int dv;
            nbr(s->chosen[l], nv, dv);
            ok = build_chain(l, nv, dv);
        }
        if (ok) {
            start_level(d);
            ok = s->end[d] == rend;
        }
        if (!ok) {
            // the rebuilt loop differs from the published one: the slice is lost
            if (lane == 0) record_check(kErrDonation, h, p, d, lo, hi, rend);
            __syncwarp();
            return true;
        }
        if (lane == 0) {
            s->idx[d] = lo;
            s->end[d] = hi;
            s->dslot[d] = h;
            s->dgen[d] = gen;
            s->downer[d] = 0;
        }
        __syncwarp();
        const __int128 acc = dfs_levels(d);
        if (lane == 0 && acc != 0) add128(out + 2 * p, acc);
        return true;
    }

    // After the warp's own queues: helps published loops until every warp
    // is done, or no record has had slices left for kIdleRounds scans in a
    // row (so helpers never hold SMs that blocks not yet resident need).
    __device__ void help_all(const PairDesc* pairs, int npairs, unsigned long long* out, unsigned total_warps) {
        constexpr unsigned kIdleRounds = 4096;
        unsigned idle = 0;
        for (unsigned round = 0; round < (1u << 24) && idle < kIdleRounds; ++round) {
            bool worked = false;
            for (int base = 0; base < kDonSlots; base += 32) {
                const int h = (int)((gw * 37 + base + lane) & (kDonSlots - 1));
                const unsigned long long w = *(volatile unsigned long long*)&don->rec[h].word;
                const bool live = (w & 0xffffffu) < ((w >> 24) & 0xffffffu);
                unsigned m = __ballot_sync(kFull, live);
                while (m) {
                    const int j = __ffs(m) - 1;
                    m &= m - 1;
                    const int hj = __shfl_sync(kFull, h, j);
                    const unsigned long long wj = __shfl_sync(kFull, w, j);
                    if (help_one(pairs, npairs, out, hj, (unsigned)(wj >> 48))) worked = true;
                }
            }
            if (worked) {
                idle = 0;
                continue;
            }
            if (*(volatile unsigned*)&don->finished >= total_warps) return;
            ++idle;
            __nanosleep(4000);
        }
    }

    __device__ __int128 edge_task(int v0, int v1) {
        if ((P->rmask[1] & 1u) && v1 >= v0) return 0;
        const int* n0;
        int d0;
        nbr(v0, n0, d0);
        set_chosen(0, v0);
        if (!build_chain(0, n0, d0)) return 0;
        const int* n1;
        int d1;
        nbr(v1, n1, d1);
        if (kBytes) bytes += 16;
        if (P->L == 1) return tail_with_candidate(v1, n1, d1);
        if (!build_chain(1, n1, d1)) return 0;
        set_chosen(1, v1);
        return dfs_from_2();
    }

    __device__ __int128 root_task(int v0) {
        const int* n0;
        int d0;
        nbr(v0, n0, d0);
        if (kBytes) bytes += 8;
        set_chosen(0, v0);
        if (!build_chain(0, n0, d0)) return 0;
        return tail_at_T();
    }
};

template <bool kBytes>
__global__ void __launch_bounds__(512, 1) match_kernel(const PairDesc* __restrict__ pairs, int npairs,
                                                    unsigned long long* __restrict__ cursors,
                                                    unsigned long long* __restrict__ out, int* __restrict__ scratch_all,
                                                    long long scratch_per_warp, int chunk,
                                                    const unsigned long long* __restrict__ params,
                                                    int leaf_on, int stage_cap, int pair_on,
                                                    unsigned long long* __restrict__ pair_tables, int pair_log2,
                                                    DonationArea* don, int split_min,
                                                    unsigned long long* __restrict__ stats) {
    // params[0] = stripes, params[1] = stripe (device memory, so a captured
    // graph can replay with new values)
    const unsigned long long stripes = params[0], stripe = params[1];
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const long long gw = (long long)blockIdx.x * nwarps + wid;
    WarpCtx<kBytes> w;
    w.s = reinterpret_cast<WarpState*>(smem_raw) + wid;
    w.stage = reinterpret_cast<int*>(reinterpret_cast<WarpState*>(smem_raw) + nwarps) + (size_t)wid * 2 * stage_cap;
    w.stage_cap = stage_cap;
    w.leaf_on = leaf_on;
    w.pair_on = pair_on && pair_tables != nullptr;
    w.pmask = (1u << pair_log2) - 1u;
    w.ptab = pair_tables ? pair_tables + ((size_t)gw << pair_log2) : nullptr;
    if (lane == 0) w.s->epoch = 0;  // the first pair sum clears the table
    w.scratch = scratch_all + gw * scratch_per_warp;
    w.lane = lane;
    w.bytes = 0;
    w.don = don;
    w.split_min = split_min;
    w.gw = gw;
    for (int p = 0; p < npairs; ++p) {
        const PairDesc pd = pairs[p];
        w.P = pd.plan;
        w.g = pd.g;
        w.cap = pd.cap;
        w.pair_idx = p;
        const int T = w.P->T;
        __int128 acc = 0;
        int cur_v0 = -1;
        unsigned cur_lo = 0, cur_hi = 0;
        for (;;) {
            // Stripe `stripe` holds the tasks t with t mod stripes == stripe;
            // grab q takes its members i in [q*chunk, q*chunk + chunk), i.e.
            // tasks i*stripes + stripe (so the stripe does not depend on chunk).
            unsigned long long q = 0;
            if (lane == 0) q = atomicAdd(&cursors[p], 1ull);
            q = __shfl_sync(kFull, q, 0);
            const unsigned long long i0 = q * (unsigned long long)chunk;
            if (i0 * stripes + stripe >= pd.ntasks) break;
            for (unsigned long long i = i0; i < i0 + (unsigned long long)chunk; ++i) {
                const unsigned long long t = i * stripes + stripe;
                if (t >= pd.ntasks) break;
                if (T == 1) {
                    acc += w.root_task((int)t);
                    continue;
                }
                const unsigned e = (unsigned)t;
                if (cur_v0 < 0 || e < cur_lo || e >= cur_hi) {
                    // last v with rowptr[v] <= e
                    int lo = 0, hi = pd.g.v_cnt;
                    while (lo < hi) {
                        int mid = (lo + hi + 1) >> 1;
                        if (pd.g.rowptr[mid] <= e) lo = mid;
                        else hi = mid - 1;
                    }
                    cur_v0 = lo;
                    cur_lo = pd.g.rowptr[lo];
                    cur_hi = pd.g.rowptr[lo + 1];
                }
                acc += w.edge_task(cur_v0, pd.g.col[e]);
            }
        }
        if (lane == 0 && acc != 0) add128(out + 2 * p, acc);
    }
    if (don) {
        if (lane == 0) {
            __threadfence();
            atomicAdd(&don->finished, 1u);
        }
        __syncwarp();
        w.help_all(pairs, npairs, out, gridDim.x * (unsigned)nwarps);
    }
    if (kBytes && lane == 0 && w.bytes) atomicAdd(stats, w.bytes);
}

// Triangle count: sum over v, u in N(v) with u < v of |N(v) ∩ N(u) ∩ [0, u)|
// (Graph::tc_mt / intersection_size_clique, src/graph.cpp:66-95,121-139).
__global__ void __launch_bounds__(256) tc_kernel(GraphView g, unsigned long long* __restrict__ cursor,
                                                 unsigned long long* __restrict__ out, int chunk) {
    const int lane = threadIdx.x & 31;
    unsigned long long acc = 0;
    int cur_v = -1;
    unsigned cur_lo = 0, cur_hi = 0;
    for (;;) {
        unsigned long long t0 = 0;
        if (lane == 0) t0 = atomicAdd(cursor, (unsigned long long)chunk);
        t0 = __shfl_sync(kFull, t0, 0);
        if (t0 >= g.e_cnt) break;
        const unsigned long long t1 = min(t0 + (unsigned long long)chunk, g.e_cnt);
        for (unsigned long long t = t0; t < t1; ++t) {
            const unsigned e = (unsigned)t;
            if (cur_v < 0 || e < cur_lo || e >= cur_hi) {
                int lo = 0, hi = g.v_cnt;
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (g.rowptr[mid] <= e) lo = mid;
                    else hi = mid - 1;
                }
                cur_v = lo;
                cur_lo = g.rowptr[lo];
                cur_hi = g.rowptr[lo + 1];
            }
            const int u = g.col[e];
            if ((unsigned)u >= (unsigned)g.v_cnt) {
                if (lane == 0) record_check(kErrBadVertex, e, u, cur_v, g.v_cnt, 0, 0);
                continue;
            }
            if (u >= cur_v) continue;
            const unsigned ub = g.rowptr[u], ue = g.rowptr[u + 1];
            acc += (unsigned long long)isect_count(g.col + cur_lo, (int)(cur_hi - cur_lo), g.col + ub, (int)(ue - ub), u,
                                                   nullptr, 0, lane);
        }
    }
    if (lane == 0 && acc) atomicAdd(out, acc);
}

// CSR checks: offsets monotone, ids in range, rows strictly increasing, no
// self loops, every edge present in both directions.
__global__ void validate_kernel(GraphView g, unsigned* __restrict__ flags) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    unsigned bad = 0;
    for (long long v = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); v < g.v_cnt; v += warps) {
        const unsigned a = g.rowptr[v], b = g.rowptr[v + 1];
        if (b < a || b > g.e_cnt) {
            bad |= 1;
            continue;
        }
        for (unsigned k = a + lane; k < b; k += 32) {
            const int x = g.col[k];
            if (x < 0 || x >= g.v_cnt) {
                bad |= 2;
                continue;
            }
            if (x == (int)v) bad |= 4;
            if (k > a && g.col[k - 1] >= x) bad |= 8;
            const unsigned xa = g.rowptr[x], xb = g.rowptr[x + 1];
            if (xb < xa || xb > g.e_cnt) {
                bad |= 1;
                continue;
            }
            const int p = lower_bound_u(g.col + xa, (int)(xb - xa), (int)v);
            if (p >= (int)(xb - xa) || g.col[xa + p] != (int)v) bad |= 16;
        }
    }
    if (bad) atomicOr(flags, bad);
}

__global__ void degree_keys_kernel(const unsigned* __restrict__ rowptr, int v_cnt, unsigned* __restrict__ keys,
                                   int* __restrict__ ids) {
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < v_cnt; v += (long long)gridDim.x * blockDim.x) {
        keys[v] = ~(rowptr[v + 1] - rowptr[v]);  // descending degree
        ids[v] = (int)v;
    }
}

__global__ void relabel_maps_kernel(const unsigned* __restrict__ rowptr, const int* __restrict__ order, int v_cnt,
                                    int* __restrict__ new_id, unsigned* __restrict__ new_deg) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i <= v_cnt; i += (long long)gridDim.x * blockDim.x) {
        if (i == v_cnt) {
            new_deg[i] = 0;
            continue;
        }
        const int o = order[i];
        new_id[o] = (int)i;
        new_deg[i] = rowptr[o + 1] - rowptr[o];
    }
}

__global__ void relabel_fill_kernel(const unsigned* __restrict__ rowptr, const int* __restrict__ col,
                                    const int* __restrict__ order, const int* __restrict__ new_id,
                                    const unsigned* __restrict__ new_rowptr, int v_cnt, int* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const long long warps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long i = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < v_cnt; i += warps) {
        const int o = order[i];
        const unsigned a = rowptr[o], b = rowptr[o + 1], dst = new_rowptr[i];
        for (unsigned k = a + lane; k < b; k += 32) out[dst + (k - a)] = new_id[col[k]];
    }
}

// ---------------------------------------------------------------------------
// host side

struct DeviceCtx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    std::mutex mu;
};

static thread_local int t_device = 0;
static thread_local double t_ms = 0;
static thread_local int64_t t_launches = 0;
static thread_local uint64_t t_bytes = 0;

static DeviceCtx* get_ctx(int* err) {
    static std::mutex mu;
    static DeviceCtx* ctxs[64] = {nullptr};
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        set_error("no CUDA device available (%s)", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
        *err = GPM_ERR_NO_DEVICE;
        return nullptr;
    }
    if (t_device < 0 || t_device >= n || t_device >= 64) {
        set_error("device %d not present", t_device);
        *err = GPM_ERR_NO_DEVICE;
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(mu);
    DeviceCtx*& c = ctxs[t_device];
    if (!c) {
        DeviceCtx* nc = new DeviceCtx();
        nc->device = t_device;
        if (cudaSetDevice(t_device) != cudaSuccess ||
            cudaDeviceGetAttribute(&nc->num_sms, cudaDevAttrMultiProcessorCount, t_device) != cudaSuccess ||
            cudaStreamCreateWithFlags(&nc->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&nc->ev0) != cudaSuccess || cudaEventCreate(&nc->ev1) != cudaSuccess) {
            set_error("CUDA initialisation failed on device %d: %s", t_device, cudaGetErrorString(cudaGetLastError()));
            delete nc;
            *err = GPM_ERR_CUDA;
            return nullptr;
        }
        c = nc;
    }
    if (cudaSetDevice(t_device) != cudaSuccess) {
        set_error("cudaSetDevice(%d) failed", t_device);
        *err = GPM_ERR_CUDA;
        return nullptr;
    }
    *err = GPM_OK;
    return c;
}

static int ensure_scratch(DeviceCtx* c, size_t bytes) {
    if (c->scratch_bytes >= bytes) return GPM_OK;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    GPM_CK(cudaMalloc(&c->scratch, bytes));
    c->scratch_bytes = bytes;
    return GPM_OK;
}

// RAII device buffer for one call
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

// Reports (and clears) an internal-check record left by a kernel.
static int take_check(const char* where) {
    unsigned long long rec[8] = {0};
    GPM_CK(cudaMemcpyFromSymbol(rec, g_check, sizeof rec));
    if (rec[0] == 0) return GPM_OK;
    const unsigned long long zero[8] = {0};
    cudaMemcpyToSymbol(g_check, zero, sizeof zero);
    set_error("%s: internal check %llu failed (values %lld %lld %lld %lld %lld %lld)", where, rec[0], (long long)rec[1],
              (long long)rec[2], (long long)rec[3], (long long)rec[4], (long long)rec[5], (long long)rec[6]);
    return GPM_ERR_CUDA;
}

static unsigned validate_csr(DeviceCtx* c, const GraphView& v, int* rc);

static int relabel_graph(DeviceCtx* c, gpm_graph* g, bool relabel) {
    const int V = g->v_cnt;
    const unsigned E = (unsigned)g->e_cnt;
    cudaStream_t st = c->stream;
    DevBuf keys, keys2, ids, order, tmp;
    GPM_CK(cudaMalloc(&keys.p, sizeof(unsigned) * (size_t)std::max(V, 1)));
    GPM_CK(cudaMalloc(&keys2.p, sizeof(unsigned) * (size_t)std::max(V, 1)));
    GPM_CK(cudaMalloc(&ids.p, sizeof(int) * (size_t)std::max(V, 1)));
    GPM_CK(cudaMalloc(&order.p, sizeof(int) * (size_t)std::max(V, 1)));
    const int threads = 256, blocks = c->num_sms * 8;
    degree_keys_kernel<<<blocks, threads, 0, st>>>(g->rowptr, V, (unsigned*)keys.p, (int*)ids.p);
    GPM_CK(cudaGetLastError());
    size_t tb = 0;
    GPM_CK(cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned*)keys.p, (unsigned*)keys2.p, (int*)ids.p,
                                           (int*)order.p, V, 0, 32, st));
    GPM_CK(cudaMalloc(&tmp.p, std::max<size_t>(tb, 1)));
    GPM_CK(cub::DeviceRadixSort::SortPairs(tmp.p, tb, (unsigned*)keys.p, (unsigned*)keys2.p, (int*)ids.p,
                                           (int*)order.p, V, 0, 32, st));
    unsigned top[2] = {~0u, ~0u};
    GPM_CK(cudaMemcpyAsync(top, keys2.p, sizeof(unsigned) * std::min(V, 2), cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    g->max_degree = V >= 1 ? (int)~top[0] : 0;
    g->max_isect = V >= 2 ? (int)~top[1] : g->max_degree;
    if (!relabel || V == 0 || E == 0) return GPM_OK;

    DevBuf new_id, new_deg, new_rowptr, new_col_u, new_col, tmp2;
    GPM_CK(cudaMalloc(&new_id.p, sizeof(int) * (size_t)V));
    GPM_CK(cudaMalloc(&new_deg.p, sizeof(unsigned) * ((size_t)V + 1)));
    GPM_CK(cudaMalloc(&new_rowptr.p, sizeof(unsigned) * ((size_t)V + 1)));
    GPM_CK(cudaMalloc(&new_col_u.p, sizeof(int) * (size_t)E));
    GPM_CK(cudaMalloc(&new_col.p, sizeof(int) * (size_t)E));
    relabel_maps_kernel<<<blocks, threads, 0, st>>>(g->rowptr, (const int*)order.p, V, (int*)new_id.p,
                                                    (unsigned*)new_deg.p);
    GPM_CK(cudaGetLastError());
    size_t sb = 0;
    GPM_CK(cub::DeviceScan::ExclusiveSum(nullptr, sb, (unsigned*)new_deg.p, (unsigned*)new_rowptr.p, V + 1, st));
    GPM_CK(cudaMalloc(&tmp2.p, std::max<size_t>(sb, 1)));
    GPM_CK(cub::DeviceScan::ExclusiveSum(tmp2.p, sb, (unsigned*)new_deg.p, (unsigned*)new_rowptr.p, V + 1, st));
    relabel_fill_kernel<<<blocks, threads, 0, st>>>(g->rowptr, g->col, (const int*)order.p, (const int*)new_id.p,
                                                    (const unsigned*)new_rowptr.p, V, (int*)new_col_u.p);
    GPM_CK(cudaGetLastError());
    size_t ssb = 0;
    GPM_CK(cub::DeviceSegmentedSort::SortKeys(nullptr, ssb, (const int*)new_col_u.p, (int*)new_col.p, (int64_t)E, V,
                                              (const unsigned*)new_rowptr.p, (const unsigned*)new_rowptr.p + 1, st));
    DevBuf tmp3;
    GPM_CK(cudaMalloc(&tmp3.p, std::max<size_t>(ssb, 1)));
    GPM_CK(cub::DeviceSegmentedSort::SortKeys(tmp3.p, ssb, (const int*)new_col_u.p, (int*)new_col.p, (int64_t)E, V,
                                              (const unsigned*)new_rowptr.p, (const unsigned*)new_rowptr.p + 1, st));
    GPM_CK(cudaStreamSynchronize(st));
    // the caller's ids stay resident for label-sensitive plans
    g->orig_rowptr = g->rowptr;
    g->orig_col = g->col;
    g->rowptr = (uint32_t*)new_rowptr.p;
    new_rowptr.p = nullptr;
    g->col = (int32_t*)new_col.p;
    new_col.p = nullptr;
    g->relabelled = true;
    // the relabelled copy must be as well-formed as the input
    GraphView nv;
    nv.rowptr = g->rowptr;
    nv.col = g->col;
    nv.v_cnt = g->v_cnt;
    nv.pad_ = 0;
    nv.e_cnt = g->e_cnt;
    int rc = GPM_OK;
    const unsigned flags = validate_csr(c, nv, &rc);
    if (rc) return rc;
    if (flags) {
        set_error("device relabel produced a malformed CSR (check flags 0x%x)", flags);
        return GPM_ERR_CUDA;
    }
    return GPM_OK;
}

static unsigned validate_csr(DeviceCtx* c, const GraphView& v, int* rc) {
    unsigned* d_flags = nullptr;
    unsigned flags = 0;
    *rc = GPM_OK;
    if (cudaMalloc(&d_flags, sizeof(unsigned)) != cudaSuccess) {
        set_error("validate: out of device memory");
        *rc = GPM_ERR_OOM;
        return 0;
    }
    cudaMemsetAsync(d_flags, 0, sizeof(unsigned), c->stream);
    validate_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(v, d_flags);
    cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    cudaFree(d_flags);
    if (e != cudaSuccess) {
        set_error("validate: %s", cudaGetErrorString(e));
        *rc = GPM_ERR_CUDA;
    }
    return flags;
}

static GraphView view_of(const gpm_graph* g, bool caller_ids = false) {
    GraphView v;
    v.rowptr = caller_ids && g->orig_rowptr ? g->orig_rowptr : g->rowptr;
    v.col = caller_ids && g->orig_col ? g->orig_col : g->col;
    v.v_cnt = g->v_cnt;
    v.pad_ = 0;
    v.e_cnt = g->e_cnt;
    return v;
}

struct LaunchSetup {
    std::vector<PairDesc> descs;
    long long blocks = 0;
    int wpb = 0;
    long long per_warp = 0;
    int stage_cap = 0;
    size_t smem = 0;
    int chunk = 0;
    int leaf_on = 0;
    int pair_on = 0;
    int split_min = 0;
    bool count_bytes = false;
};

constexpr int kPairLog2 = 13;  // 8192-entry table per warp

// Validates the pairs and sizes the launch from the current options.
static int prepare_pairs(DeviceCtx* c, int n, gpm_graph* const* graphs, const gpm_plan* const* plans,
                         size_t scratch_budget_extra, LaunchSetup& ls) {
    Options& o = options();
    int cap = 1, nslots = 1;
    ls.descs.assign(n, PairDesc());
    for (int i = 0; i < n; ++i) {
        const gpm_graph* g = graphs[i];
        const gpm_plan* p = plans[i];
        if (!g || !p) {
            set_error("pair %d: null graph or plan", i);
            return GPM_ERR_INVALID_ARG;
        }
        if (g->device != c->device || p->device != c->device) {
            set_error("pair %d: graph/plan live on another device", i);
            return GPM_ERR_INVALID_ARG;
        }
        PairDesc& d = ls.descs[i];
        d.g = view_of(g, p->host.label_sensitive != 0);
        d.plan = p->dev;
        d.ntasks = p->host.T == 1 ? (unsigned long long)g->v_cnt : (unsigned long long)g->e_cnt;
        // every set built is a subset of one neighbour list: the largest degree
        // bounds it (inclusion-exclusion temporaries can be N(v0) itself)
        d.cap = std::max(1, g->max_degree);
        d.pad_ = 0;
        cap = std::max(cap, d.cap);
        nslots = std::max(nslots, p->host.nslots);
    }
    ls.wpb = (int)o.warps_per_block;
    ls.stage_cap = (int)o.stage_max;
    ls.smem = sizeof(WarpState) * ls.wpb + sizeof(int) * 2 * (size_t)ls.stage_cap * ls.wpb;
    ls.count_bytes = o.count_bytes != 0;
    const void* kfn = ls.count_bytes ? (const void*)match_kernel<true> : (const void*)match_kernel<false>;
    GPM_CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls.smem));
    // a persistent grid: no more blocks than can be resident at once
    int occ = 0;
    GPM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, ls.wpb * 32, ls.smem));
    if (occ < 1) {
        set_error("launch shape does not fit an SM: %d warps per block, %zu bytes of shared memory", ls.wpb, ls.smem);
        return GPM_ERR_INVALID_ARG;
    }
    ls.blocks = (long long)c->num_sms * std::min<long long>(o.blocks_per_sm, occ);
    ls.per_warp = (long long)nslots * cap;
    // shrink the grid when the per-warp scratch would not fit in free memory
    size_t free_b = 0, total_b = 0;
    GPM_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = (size_t)((free_b + scratch_budget_extra) * 0.6);
    while (ls.blocks > 1 && (size_t)ls.blocks * ls.wpb * ls.per_warp * sizeof(int) > budget)
        ls.blocks = (ls.blocks + 1) / 2;
    const int alpha4[3] = {(int)o.merge_alpha4[0], (int)o.merge_alpha4[1], (int)o.merge_alpha4[2]};
    GPM_CK(cudaMemcpyToSymbolAsync(c_merge_alpha4, alpha4, sizeof alpha4, 0, cudaMemcpyHostToDevice, c->stream));
    ls.chunk = (int)o.chunk;
    ls.leaf_on = (int)o.leaf_batch;
    ls.pair_on = 0;
    if (o.pair_leaf) {
        bool any = false;
        for (int i = 0; i < n; ++i) any |= plans[i]->host.pair_ok && graphs[i]->v_cnt <= (1 << 24);
        ls.pair_on = any ? 1 : 0;
    }
    ls.split_min = (int)o.split;
    return GPM_OK;
}

// small device words of a launch: cursors[n], out[2n], stats[2], params[2]
static size_t small_words(int n) { return (size_t)n * 3 + 4; }

// Scratch of a launch: per-warp set slots, per-warp pair tables, then the
// donation records (zeroed before every launch).
struct ScratchLayout {
    size_t tables = 0, donation = 0, total = 0;
};

static ScratchLayout scratch_layout(const LaunchSetup& ls) {
    const size_t warps = (size_t)ls.blocks * ls.wpb;
    ScratchLayout s;
    size_t b = warps * (size_t)ls.per_warp * sizeof(int);
    b = (b + 255) & ~(size_t)255;
    s.tables = b;
    if (ls.pair_on) b += warps * ((size_t)1 << kPairLog2) * sizeof(unsigned long long);
    s.donation = b;
    if (ls.split_min > 0) b += sizeof(DonationArea);
    s.total = std::max<size_t>(b, 1);
    return s;
}

static size_t scratch_bytes(const LaunchSetup& ls) { return scratch_layout(ls).total; }

static cudaError_t enqueue_match(const LaunchSetup& ls, int n, const PairDesc* d_pairs,
                                 unsigned long long* d_small, int* scratch, cudaStream_t st) {
    unsigned long long* cursors = d_small;
    unsigned long long* out = cursors + n;
    unsigned long long* stats = out + 2 * n;
    const unsigned long long* params = stats + 2;
    const ScratchLayout lay = scratch_layout(ls);
    unsigned long long* tables = ls.pair_on ? (unsigned long long*)((char*)scratch + lay.tables) : nullptr;
    DonationArea* don = ls.split_min > 0 ? (DonationArea*)((char*)scratch + lay.donation) : nullptr;
    if (don) {
        const cudaError_t e = cudaMemsetAsync(don, 0, sizeof(DonationArea), st);
        if (e != cudaSuccess) return e;
    }
    if (ls.count_bytes)
        match_kernel<true><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(
            d_pairs, n, cursors, out, scratch, ls.per_warp, ls.chunk, params, ls.leaf_on, ls.stage_cap, ls.pair_on,
            tables, kPairLog2, don, ls.split_min, stats);
    else
        match_kernel<false><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(
            d_pairs, n, cursors, out, scratch, ls.per_warp, ls.chunk, params, ls.leaf_on, ls.stage_cap, ls.pair_on,
            tables, kPairLog2, don, ls.split_min, stats);
    return cudaGetLastError();
}

// Launches the matcher over n pairs and leaves raw 128-bit sums in host_raw
// (2 words per pair).
static int run_pairs(DeviceCtx* c, int n, gpm_graph* const* graphs, const gpm_plan* const* plans,
                     unsigned long long* host_raw) {
    LaunchSetup ls;
    int rc = prepare_pairs(c, n, graphs, plans, c->scratch_bytes, ls);
    if (rc) return rc;
    rc = ensure_scratch(c, scratch_bytes(ls));
    if (rc) return rc;
    DevBuf d_pairs, d_small;
    GPM_CK(cudaMalloc(&d_pairs.p, sizeof(PairDesc) * n));
    const size_t words = small_words(n);
    GPM_CK(cudaMalloc(&d_small.p, words * sizeof(unsigned long long)));
    cudaStream_t st = c->stream;
    std::vector<unsigned long long> init(words, 0);
    init[3 * n + 2] = (unsigned long long)options().stripes;
    init[3 * n + 3] = (unsigned long long)options().stripe;
    GPM_CK(cudaMemcpyAsync(d_pairs.p, ls.descs.data(), sizeof(PairDesc) * n, cudaMemcpyHostToDevice, st));
    GPM_CK(cudaMemcpyAsync(d_small.p, init.data(), words * sizeof(unsigned long long), cudaMemcpyHostToDevice, st));
    GPM_CK(cudaEventRecord(c->ev0, st));
    GPM_CK(enqueue_match(ls, n, (const PairDesc*)d_pairs.p, (unsigned long long*)d_small.p, (int*)c->scratch, st));
    GPM_CK(cudaEventRecord(c->ev1, st));
    std::vector<unsigned long long> raw(2 * n + 2);
    GPM_CK(cudaMemcpyAsync(raw.data(), (unsigned long long*)d_small.p + n, sizeof(unsigned long long) * (2 * n + 2),
                           cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    float ms = 0;
    GPM_CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    t_ms = ms;
    t_launches = 1;
    t_bytes = raw[2 * n];
    memcpy(host_raw, raw.data(), sizeof(unsigned long long) * 2 * n);
    return take_check("pattern matching");
}

static int finish_counts(int n, const gpm_plan* const* plans, const unsigned long long* raw, gpm_u128* outs) {
    if (options().raw_sums) {
        // undivided two's-complement sums (partial stripes are summed by the caller)
        for (int i = 0; i < n; ++i) {
            outs[i].lo = raw[2 * i];
            outs[i].hi = raw[2 * i + 1];
        }
        return GPM_OK;
    }
    if (options().stripes != 1) {
        set_error("a striped launch covers part of the work: set raw_sums=1 and divide the summed stripes");
        return GPM_ERR_INVALID_ARG;
    }
    for (int i = 0; i < n; ++i) {
        const unsigned __int128 u = ((unsigned __int128)raw[2 * i + 1] << 64) | raw[2 * i];
        const __int128 s = (__int128)u;
        if (s < 0) {
            set_error("pair %d: negative total (128-bit overflow)", i);
            return GPM_ERR_OVERFLOW;
        }
        const unsigned __int128 q = u / (unsigned __int128)plans[i]->host.redundancy;
        outs[i].lo = (uint64_t)q;
        outs[i].hi = (uint64_t)(q >> 64);
    }
    return GPM_OK;
}

}  // namespace gpm

using namespace gpm;

extern "C" {

GPM_API int gpm_set_device(int32_t device) {
    clear_error();
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        set_error("gpm_set_device: device %d not present", device);
        return GPM_ERR_NO_DEVICE;
    }
    t_device = device;
    return GPM_OK;
}

GPM_API int gpm_graph_create(int32_t v_cnt, const uint32_t* rowptr, const int32_t* col, int32_t relabel,
                             gpm_graph** out) {
    clear_error();
    if (!out || v_cnt < 1 || !rowptr) {
        set_error("gpm_graph_create: need v_cnt >= 1, rowptr and out");
        return GPM_ERR_INVALID_ARG;
    }
    *out = nullptr;
    const uint64_t E = rowptr[v_cnt];
    if (rowptr[0] != 0 || (E > 0 && !col)) {
        set_error("gpm_graph_create: rowptr[0] must be 0 and col non-null");
        return GPM_ERR_INVALID_ARG;
    }
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    gpm_graph* g = new gpm_graph();
    g->v_cnt = v_cnt;
    g->e_cnt = E;
    g->device = c->device;
    auto fail = [&](int rc) {
        if (g->orig_rowptr && g->orig_rowptr != g->rowptr) cudaFree(g->orig_rowptr);
        if (g->orig_col && g->orig_col != g->col) cudaFree(g->orig_col);
        if (g->rowptr) cudaFree(g->rowptr);
        if (g->col) cudaFree(g->col);
        delete g;
        return rc;
    };
    cudaStream_t st = c->stream;
    if (cudaMalloc(&g->rowptr, sizeof(uint32_t) * ((size_t)v_cnt + 1)) != cudaSuccess ||
        cudaMalloc(&g->col, sizeof(int32_t) * std::max<size_t>(E, 1)) != cudaSuccess) {
        set_error("gpm_graph_create: out of device memory for %llu edges", (unsigned long long)E);
        return fail(GPM_ERR_OOM);
    }
    if (cudaMemcpyAsync(g->rowptr, rowptr, sizeof(uint32_t) * ((size_t)v_cnt + 1), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        (E && cudaMemcpyAsync(g->col, col, sizeof(int32_t) * E, cudaMemcpyHostToDevice, st) != cudaSuccess)) {
        set_error("gpm_graph_create: upload failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(GPM_ERR_CUDA);
    }
    unsigned* d_flags = nullptr;
    if (cudaMalloc(&d_flags, sizeof(unsigned)) != cudaSuccess) return fail(GPM_ERR_OOM);
    cudaMemsetAsync(d_flags, 0, sizeof(unsigned), st);
    validate_kernel<<<c->num_sms * 8, 256, 0, st>>>(view_of(g), d_flags);
    unsigned flags = 0;
    cudaMemcpyAsync(&flags, d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    cudaFree(d_flags);
    if (e != cudaSuccess) {
        set_error("gpm_graph_create: validation failed: %s", cudaGetErrorString(e));
        return fail(GPM_ERR_CUDA);
    }
    if (flags) {
        set_error("gpm_graph_create: malformed CSR (%s%s%s%s%s)", flags & 1 ? "offsets " : "",
                  flags & 2 ? "ids-out-of-range " : "", flags & 4 ? "self-loops " : "",
                  flags & 8 ? "unsorted-or-duplicate " : "", flags & 16 ? "asymmetric" : "");
        return fail(GPM_ERR_INVALID_ARG);
    }
    int rc = relabel_graph(c, g, relabel != 0);
    if (rc) return fail(rc);
    *out = g;
    return GPM_OK;
}

GPM_API int gpm_graph_destroy(gpm_graph* g) {
    clear_error();
    if (!g) return GPM_OK;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(g->device);
    if (g->orig_rowptr && g->orig_rowptr != g->rowptr) cudaFree(g->orig_rowptr);
    if (g->orig_col && g->orig_col != g->col) cudaFree(g->orig_col);
    if (g->rowptr) cudaFree(g->rowptr);
    if (g->col) cudaFree(g->col);
    cudaSetDevice(dev);
    delete g;
    return GPM_OK;
}

GPM_API int gpm_graph_stats(const gpm_graph* g, int64_t* v_cnt, int64_t* e_cnt, int64_t* max_degree,
                            int64_t* max_intersection_size) {
    clear_error();
    if (!g) {
        set_error("gpm_graph_stats: null graph");
        return GPM_ERR_INVALID_ARG;
    }
    if (v_cnt) *v_cnt = g->v_cnt;
    if (e_cnt) *e_cnt = (int64_t)g->e_cnt;
    if (max_degree) *max_degree = g->max_degree;
    if (max_intersection_size) *max_intersection_size = g->max_isect;
    return GPM_OK;
}

GPM_API int gpm_tri_count(gpm_graph* g, uint64_t* out) {
    clear_error();
    if (!g || !out) {
        set_error("gpm_tri_count: null argument");
        return GPM_ERR_INVALID_ARG;
    }
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    DevBuf buf;
    GPM_CK(cudaMalloc(&buf.p, 2 * sizeof(unsigned long long)));
    cudaStream_t st = c->stream;
    GPM_CK(cudaMemsetAsync(buf.p, 0, 2 * sizeof(unsigned long long), st));
    unsigned long long* d = (unsigned long long*)buf.p;
    GPM_CK(cudaEventRecord(c->ev0, st));
    tc_kernel<<<c->num_sms * 8, 256, 0, st>>>(view_of(g), d, d + 1, (int)options().chunk);
    GPM_CK(cudaGetLastError());
    GPM_CK(cudaEventRecord(c->ev1, st));
    unsigned long long h[2];
    GPM_CK(cudaMemcpyAsync(h, d, sizeof h, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    t_ms = ms;
    t_launches = 1;
    t_bytes = 0;
    int rc = take_check("gpm_tri_count");
    if (rc) return rc;
    *out = h[1];
    return GPM_OK;
}

GPM_API int gpm_plan_create(const int64_t* tables, int32_t n_words, gpm_plan** out) {
    clear_error();
    if (!out) return GPM_ERR_INVALID_ARG;
    *out = nullptr;
    DevPlan hp;
    int rc = compile_plan(tables, n_words, &hp);
    if (rc) return rc;
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    gpm_plan* p = new gpm_plan();
    p->host = hp;
    p->device = c->device;
    if (cudaMalloc(&p->dev, sizeof(DevPlan)) != cudaSuccess ||
        cudaMemcpy(p->dev, &hp, sizeof(DevPlan), cudaMemcpyHostToDevice) != cudaSuccess) {
        set_error("gpm_plan_create: %s", cudaGetErrorString(cudaGetLastError()));
        if (p->dev) cudaFree(p->dev);
        delete p;
        return GPM_ERR_CUDA;
    }
    *out = p;
    return GPM_OK;
}

GPM_API int gpm_plan_destroy(gpm_plan* p) {
    clear_error();
    if (!p) return GPM_OK;
    if (p->dev) cudaFree(p->dev);
    delete p;
    return GPM_OK;
}

GPM_API int gpm_batch_count(int32_t n_pairs, gpm_graph* const* graphs, const gpm_plan* const* plans, gpm_u128* outs) {
    clear_error();
    if (n_pairs < 1 || !graphs || !plans || !outs) {
        set_error("gpm_batch_count: need n_pairs >= 1 and non-null arrays");
        return GPM_ERR_INVALID_ARG;
    }
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    std::vector<unsigned long long> raw(2 * (size_t)n_pairs);
    int rc = run_pairs(c, n_pairs, graphs, plans, raw.data());
    if (rc) return rc;
    return finish_counts(n_pairs, plans, raw.data(), outs);
}

GPM_API int gpm_count(gpm_graph* g, const gpm_plan* p, gpm_u128* out) {
    gpm_graph* gs[1] = {g};
    const gpm_plan* ps[1] = {p};
    return gpm_batch_count(1, gs, ps, out);
}

GPM_API int gpm_count_host(int32_t v_cnt, const uint32_t* rowptr, const int32_t* col, int32_t n_plans,
                           const int64_t* tables, const int32_t* n_words, gpm_u128* outs) {
    clear_error();
    if (n_plans < 1 || !tables || !n_words || !outs) {
        set_error("gpm_count_host: need n_plans >= 1 and non-null arrays");
        return GPM_ERR_INVALID_ARG;
    }
    gpm_graph* g = nullptr;
    int rc = gpm_graph_create(v_cnt, rowptr, col, 1, &g);
    if (rc) return rc;
    std::vector<gpm_plan*> plans(n_plans, nullptr);
    size_t off = 0;
    for (int i = 0; i < n_plans && rc == GPM_OK; ++i) {
        rc = gpm_plan_create(tables + off, n_words[i], &plans[i]);
        off += (size_t)n_words[i];
    }
    if (rc == GPM_OK) {
        std::vector<gpm_graph*> gs(n_plans, g);
        std::vector<const gpm_plan*> ps(plans.begin(), plans.end());
        rc = gpm_batch_count(n_plans, gs.data(), ps.data(), outs);
    }
    std::string msg = rc ? gpm_last_error() : std::string();
    for (gpm_plan* p : plans) gpm_plan_destroy(p);
    gpm_graph_destroy(g);
    if (rc) set_error("%s", msg.c_str());
    return rc;
}

struct gpm_batch_exec {
    int n = 0;
    int device = 0;
    std::vector<const gpm_plan*> plans;
    LaunchSetup ls;
    void* d_pairs = nullptr;
    unsigned long long* d_small = nullptr;
    unsigned long long* h_small = nullptr;  // pinned: out[2n], stats[2], params[2]
    int* scratch = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~gpm_batch_exec() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (d_pairs) cudaFree(d_pairs);
        if (d_small) cudaFree(d_small);
        if (h_small) cudaFreeHost(h_small);
        if (scratch) cudaFree(scratch);
    }
};

// Builds the replayable graph: params H2D, zero the counters, the
// persistent launch, results D2H.  The exec owns its buffers so other calls
// cannot move them between replays.
static int exec_build(DeviceCtx* c, gpm_batch_exec* e, gpm_graph* const* graphs) {
    const int n = e->n;
    int rc = prepare_pairs(c, n, graphs, e->plans.data(), 0, e->ls);
    if (rc) return rc;
    const size_t words = small_words(n);
    GPM_CK(cudaMalloc(&e->d_pairs, sizeof(PairDesc) * n));
    GPM_CK(cudaMalloc(&e->d_small, words * sizeof(unsigned long long)));
    GPM_CK(cudaMallocHost(&e->h_small, (2 * (size_t)n + 4) * sizeof(unsigned long long)));
    GPM_CK(cudaMalloc(&e->scratch, scratch_bytes(e->ls)));
    cudaStream_t st = c->stream;
    GPM_CK(cudaMemcpyAsync(e->d_pairs, e->ls.descs.data(), sizeof(PairDesc) * n, cudaMemcpyHostToDevice, st));
    GPM_CK(cudaStreamSynchronize(st));
    unsigned long long* h_params = e->h_small + 2 * n + 2;
    unsigned long long* d_params = e->d_small + 3 * n + 2;
    GPM_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    cudaMemcpyAsync(d_params, h_params, 2 * sizeof(unsigned long long), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(e->d_small, 0, (3 * (size_t)n + 2) * sizeof(unsigned long long), st);
    const cudaError_t qe = enqueue_match(e->ls, n, (const PairDesc*)e->d_pairs, e->d_small, e->scratch, st);
    cudaMemcpyAsync(e->h_small, e->d_small + n, (2 * (size_t)n + 2) * sizeof(unsigned long long),
                    cudaMemcpyDeviceToHost, st);
    cudaGraph_t g = nullptr;
    cudaError_t err = cudaStreamEndCapture(st, &g);
    if (err == cudaSuccess && qe != cudaSuccess) err = qe;
    if (err != cudaSuccess) {
        set_error("CUDA graph capture failed: %s", cudaGetErrorString(err));
        if (g) cudaGraphDestroy(g);
        return GPM_ERR_CUDA;
    }
    e->graph = g;
    GPM_CK(cudaGraphInstantiate(&e->exec, g, 0));
    return GPM_OK;
}

GPM_API int gpm_batch_exec_run(gpm_batch_exec** exec, int32_t n_pairs, gpm_graph* const* graphs,
                               const gpm_plan* const* plans, gpm_u128* outs) {
    clear_error();
    if (!exec || n_pairs < 1 || !graphs || !plans || !outs) {
        set_error("gpm_batch_exec_run: need n_pairs >= 1 and non-null arrays");
        return GPM_ERR_INVALID_ARG;
    }
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!*exec) {
        gpm_batch_exec* e = new gpm_batch_exec();
        e->n = n_pairs;
        e->device = c->device;
        e->plans.assign(plans, plans + n_pairs);
        int rc = exec_build(c, e, graphs);
        if (rc) {
            delete e;
            return rc;
        }
        *exec = e;
    }
    gpm_batch_exec* e = *exec;
    if (e->n != n_pairs || e->device != c->device) {
        set_error("gpm_batch_exec_run: exec was built for %d pairs on device %d", e->n, e->device);
        return GPM_ERR_INVALID_ARG;
    }
    const int n = e->n;
    e->h_small[2 * n + 2] = (unsigned long long)options().stripes;
    e->h_small[2 * n + 3] = (unsigned long long)options().stripe;
    cudaStream_t st = c->stream;
    GPM_CK(cudaEventRecord(c->ev0, st));
    GPM_CK(cudaGraphLaunch(e->exec, st));
    GPM_CK(cudaEventRecord(c->ev1, st));
    GPM_CK(cudaStreamSynchronize(st));
    float ms = 0;
    GPM_CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    t_ms = ms;
    t_launches = 1;
    t_bytes = e->h_small[2 * n];
    std::vector<unsigned long long> raw(e->h_small, e->h_small + 2 * n);
    int rc = take_check("gpm_batch_exec_run");
    if (rc) return rc;
    return finish_counts(n, e->plans.data(), raw.data(), outs);
}

GPM_API int gpm_batch_exec_destroy(gpm_batch_exec* exec) {
    delete exec;
    return GPM_OK;
}

GPM_API int gpm_last_launch_stats(double* kernel_ms, int64_t* launches, uint64_t* algo_bytes) {
    if (kernel_ms) *kernel_ms = t_ms;
    if (launches) *launches = t_launches;
    if (algo_bytes) *algo_bytes = t_bytes;
    return GPM_OK;
}

}  // extern "C"
