// Device core of the matcher: the per-warp DFS (WarpCtx) and the persistent
// match_kernel, included by gpm_device.cu inside namespace gpm.
//
// With GPM_EMU defined, the same source compiles as host C++ against the
// warp emulator of the tests (tests/emu/warp_emu.h: 32 host threads per warp,
// lock-step warp intrinsics), so the kernel's indexing and its donation
// protocol can be checked on the CPU under AddressSanitizer.
#pragma once
constexpr unsigned kFull = 0xffffffffu;

// Internal-check record: the first kernel that detects an impossible state
// (a merge window that does not advance, an id outside the graph) writes a
// code and a few values here and skips the work; the host reports it.
// [0] code, [1..7] values.
constexpr int kErrMergeStall = 1, kErrBadVertex = 2, kErrLoopIndex = 5, kErrSetSize = 6, kErrStage = 7;

// Ints per stage region of a warp: the staging capacity rounded up to 16
// bytes plus 8 ints, so that a bulk copy of a 16-byte aligned span around a
// set of stage_cap ints fits.
__host__ __device__ constexpr int stage_stride(int stage_cap) { return ((stage_cap + 3) & ~3) + 8; }
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

struct alignas(16) WarpState {
    unsigned long long mbar;  // mbarrier of this warp's bulk copies into its stage
    unsigned mphase;          // parity of the mbarrier's current phase
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
// list elements (candidate degrees) one loop slice covers at most, unless it
// is a single candidate
constexpr unsigned kLoopBudget = 16384;
constexpr int kErrDonation = 4;

// Record kinds: a loop of depth d, the batched deepest level (taken in
// coarser slices), and the two phases of a shared pair sum: filling the
// owner's table from the smaller side's candidates, then probing it with the
// other side's (the owner waits until every slice of a phase is done).
constexpr int kDonLoop = 0, kDonLeaf = 1, kDonPairFill = 2, kDonPairProbe = 3;
// pair sums too big for a warp's table: a dense per-vertex counter array
// from the pool, filled, probed and cleared again in three shared phases
constexpr int kDonDenseFill = 4, kDonDenseProbe = 5, kDonDenseClear = 6;
// the first phase of a long pair sum: the candidates' list lengths below the
// bound, in blocks of 32 candidates (the element phases are sliced by them)
constexpr int kDonPairLen = 7;
__device__ __forceinline__ bool don_pair_kind(int kind) { return (kind & 0xff) >= kDonPairFill && (kind & 0xff) <= kDonPairLen; }
__device__ __forceinline__ bool don_dense_kind(int kind) { return (kind & 0xff) >= kDonDenseFill && (kind & 0xff) <= kDonDenseClear; }
// the pass a pair-sum element phase runs: 0 insert / count, 1 probe / sum, 2 clear
__device__ __forceinline__ int don_phase(int kind) {
    const int k = kind & 0xff;
    return (k == kDonPairFill || k == kDonDenseFill) ? 0 : ((k == kDonPairProbe || k == kDonDenseProbe) ? 1 : 2);
}
// pair-sum element phases: the phase runs over side A (level L-1); bits 16+
// hold log2 of the elements per unit
constexpr int kDonSideA = 0x100;

// Pair sums share their length phase from this many blocks of 32 candidates
// on, and slice their element phases in units of 2^GPM_PAIR_UNIT_LOG2
// elements (the emulated-warp tests build with 1 and 0: every phase shared,
// one-element units).
#ifndef GPM_PAIR_SHARE_BLOCKS
#define GPM_PAIR_SHARE_BLOCKS 8
#endif
#ifndef GPM_PAIR_UNIT_LOG2
#define GPM_PAIR_UNIT_LOG2 6
#endif

// Words of each warp's scratch tail that hold a pair sum's block sums per
// side (one word per 32 candidates of a list of at most cap).
__host__ __device__ constexpr long long pair_bs_stride(long long cap) { return ((cap + 31) / 32 + 4) & ~3ll; }

struct Donation {
    unsigned long long word;  // generation (16 bits) | end (24) | next (24)
    int pair;
    int depth;
    int chosen[kMaxN];  // pair sums: chosen[0, L-1), and in the last word the phase side's candidate count
    int kind;        // kDon*
    int owner;       // pair sums: global warp index of the owner (its arrays and table)
    unsigned epoch;  // pair sums: tag of the owner's live table entries, or the dense array's index
    unsigned done;   // pair sums: units of the phase finished
};
static_assert(sizeof(Donation) == 64, "one record per 64 bytes");

struct DonationArea {
    Donation rec[kDonSlots];
    unsigned busy[kDonSlots];    // 1 while a record's owner holds the slot
    unsigned visits[kDonSlots];  // helpers that may still claim from a record
    unsigned finished;           // warps done with their own queues
    unsigned held;               // slots held by owners (records that may be live)
    unsigned pad_[2];
};

// Claims are fetch-and-adds on the record word's next field, so that any
// number of warps can take slices of one record at once (a compare-and-swap
// per claim let one claim through per round trip while every other warp
// retried).  An add cannot check the generation first, so a warp registers
// as a visitor of the record (visits[h]) before it reads the word and stays
// one until it stops claiming; an owner publishes a new generation in a
// record only when it has no visitors: a slot is taken only if unvisited,
// and a pair sum waits for its helpers to leave between phases.  So every
// add lands in the generation its warp checked.  The next field may run
// past end by one slice per claimer; end stays below kDonEndMax so that it
// never carries into end.
constexpr unsigned kDonEndMax = 0xf00000u;

__device__ __forceinline__ unsigned long long don_pack(unsigned gen, unsigned end, unsigned next) {
    return ((unsigned long long)(gen & 0xffffu) << 48) | ((unsigned long long)(end & 0xffffffu) << 24) |
           (unsigned long long)(next & 0xffffffu);
}

// Adds take to record r's next field (the caller visits r and has seen
// generation gen in it); returns the slice [lo, hi), empty when the record
// was exhausted.
__device__ void don_take(Donation* r, unsigned gen, unsigned take, int& lo, int& hi) {
    lo = hi = 0;
    const unsigned long long old = atomicAdd(&r->word, (unsigned long long)take);
    const unsigned end = (unsigned)(old >> 24) & 0xffffffu, next = (unsigned)old & 0xffffffu;
    if ((unsigned)(old >> 48) != (gen & 0xffffu) || next + take > 0xffffffu) {
        record_check(kErrDonation, gen, (long long)old, take, 0, 0, 5);
        return;
    }
    if (next >= end) return;
    lo = (int)next;
    hi = (int)min(next + take, end);
}

// Takes the next slice of record r (generation gen, visited by the caller);
// lo == hi when the record is exhausted or holds another generation.  A
// slice is 1/32 of what is left, within the bounds of the record's kind: a
// loop's first slice for a helper one candidate (its later slices are
// weighted by claim_more), batched leaves [8, 128], pair-sum lengths [1, 16]
// blocks of 32 candidates, pair-sum element phases [1, 64] units (of 64
// elements or more).
__device__ void don_claim(Donation* r, unsigned gen, int kind, int& lo, int& hi) {
    lo = hi = 0;
    const unsigned long long w = *(volatile unsigned long long*)&r->word;
    if ((unsigned)(w >> 48) != (gen & 0xffffu)) return;
    const unsigned end = (unsigned)(w >> 24) & 0xffffffu, next = (unsigned)w & 0xffffffu;
    if (next >= end) return;
    kind &= 0xff;
    const unsigned smin = kind == kDonLeaf ? 8u : 1u;
    const unsigned smax = kind == kDonLeaf ? 128u : (kind == kDonLoop ? 1u : (kind == kDonPairLen ? 16u : 64u));
    const unsigned take = min(end - next, min(smax, max(smin, (end - next) >> 5)));
    don_take(r, gen, take, lo, hi);
}

// A free, unvisited slot (lane 0): busy is taken, then the slot is given up
// again if some warp may still claim from its last record.
__device__ int don_take_slot(DonationArea* don, long long seed) {
    for (int probe = 0; probe < 4; ++probe) {
        const int c = (int)((seed + probe * 257) & (kDonSlots - 1));
        if (atomicCAS(&don->busy[c], 0u, 1u) != 0u) continue;
        __threadfence();
        if (atomicAdd(&don->visits[c], 0u) == 0u) return c;
        atomicExch(&don->busy[c], 0u);
    }
    return -1;
}

// A helper's visit of record h: registered before it reads the record
__device__ __forceinline__ void don_visit(DonationArea* don, int h) {
    atomicAdd(&don->visits[h], 1u);
    __threadfence();
}
__device__ __forceinline__ void don_leave(DonationArea* don, int h) {
    __threadfence();
    atomicAdd(&don->visits[h], ~0u);  // minus one
}

__device__ __forceinline__ unsigned lanemask_lt() {
#ifdef GPM_EMU
    return (1u << (threadIdx.x & 31u)) - 1u;
#else
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
#endif
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

// Merge variant with 128-bit window loads: each lane loads 4 consecutive
// ints of B (one 16-byte load), so a step sees a 128-element window of B
// against 32 elements of A.  The window starts at the 16-byte boundary at or
// below B + j; its elements before j (already consumed, all below every
// remaining A element) read as INT_MIN and are never counted, elements at or
// past nb read as INT_MAX, and a lane whose 4 ints would cross nb loads them
// one by one, so nothing past the list is read.  Each lane finds its A
// element in the window: a 5-step shuffle search over the lanes' first
// elements, then a look at that lane's 4 (and the next lane's first).  Used
// when c_merge_vec is 1.
template <bool kStore>
__device__ int warp_merge4(const int* A, int na, const int* B, int nb, int* out, const int* chosen, int nch,
                           int lane) {
    int i = 0, j = 0, acc = 0;
    while (i < na && j < nb) {
        const int a = (i + lane < na) ? A[i + lane] : INT_MAX;
        const int sh = (int)(((unsigned long long)(B + j) >> 2) & 3ull);
        const int jb = j - sh;  // B + jb is 16-byte aligned
        const int k0 = jb + 4 * lane;
        int b[4];
        if (k0 >= j && k0 + 3 < nb) {
#ifdef GPM_EMU
            for (int t = 0; t < 4; ++t) b[t] = B[k0 + t];
#else
            const int4 q = *reinterpret_cast<const int4*>(B + k0);
            b[0] = q.x;
            b[1] = q.y;
            b[2] = q.z;
            b[3] = q.w;
#endif
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int k = k0 + t;
                b[t] = k < j ? INT_MIN : (k < nb ? B[k] : INT_MAX);
            }
        }
        // last lane whose first element is below a, then inside its four
        int pos = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const int f = __shfl_sync(kFull, b[0], pos + step);
            if (pos + step < 32 && f < a) pos += step;
        }
        const int q0 = __shfl_sync(kFull, b[0], pos), q1 = __shfl_sync(kFull, b[1], pos),
                  q2 = __shfl_sync(kFull, b[2], pos), q3 = __shfl_sync(kFull, b[3], pos);
        const int nxt = __shfl_sync(kFull, b[0], (pos + 1) & 31);
        bool found = (a != INT_MAX) &&
                     (q0 == a || q1 == a || q2 == a || q3 == a || (pos < 31 && nxt == a));
        if (!kStore && found)
            for (int c = 0; c < nch; ++c)
                if (chosen[c] == a) found = false;
        const unsigned fm = __ballot_sync(kFull, found);
        if (kStore && found) out[acc + __popc(fm & lanemask_lt())] = a;
        acc += __popc(fm);
        // consume A elements <= the window's last real element and B
        // elements <= the A window's largest
        int wlast = INT_MIN;
#pragma unroll
        for (int t = 0; t < 4; ++t)
            if (k0 + t >= j && k0 + t < nb) wlast = max(wlast, b[t]);
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) wlast = max(wlast, __shfl_xor_sync(kFull, wlast, o));
        const int amax = __shfl_sync(kFull, a, 31);
        int mine = 0;
#pragma unroll
        for (int t = 0; t < 4; ++t) mine += (k0 + t >= j && k0 + t < nb && b[t] <= amax) ? 1 : 0;
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) mine += __shfl_xor_sync(kFull, mine, o);
        const int di = __popc(__ballot_sync(kFull, a <= wlast));
        const int dj = mine;
        if (di == 0 && dj == 0) {
            const int a0 = __shfl_sync(kFull, a, 0);
            if (lane == 0) record_check(kErrMergeStall, na, nb, i, j, a0, wlast);
            break;
        }
        i += di;
        j += dj;
    }
    if (kStore) __syncwarp();
    return acc;
}

// 1: merges read B through 128-bit windows (warp_merge4); 0: one int per lane.
__constant__ int c_merge_vec = 1;

// Merge when both lists are of similar length: a binary-search round costs
// about log2(nb) dependent loads for 32 elements of the short list, a merge
// step one coalesced load per list for at least 32 elements.
// alpha4 = 4 x the weight of a binary-search round, per bucket of the longer
// list's length (< 256, < 8192, larger); the autotuner sets them.
__constant__ int c_merge_alpha4[3] = {4, 4, 4};

// Longest pair sum (elements of both sides' lists) one warp takes on; a
// longer one runs as loops, which donation spreads over idle warps (0: no cap).
__constant__ long long c_pair_max_ops = 0;

__device__ __forceinline__ bool prefer_merge(int na, int nb) {
    const int lg = 32 - __clz(nb | 1);
    const int a4 = c_merge_alpha4[nb < 256 ? 0 : (nb < 8192 ? 1 : 2)];
    return (long long)na * lg * a4 >= 4ll * (long long)(na + nb);
}

// Warp galloping search: the position of the first element >= x in
// B[lo, nb), for 32 keys at once (one per lane, ascending across lanes).
// Lane i probes B[lo + 2^i - 1] — the whole exponential probe sequence in
// one round of loads — then each lane finds its bracket among the probes
// with a 5-step shuffle search and binary-searches inside it:
// about log2(distance from lo) dependent loads instead of log2(nb - lo).
// Every lane must call it (it shuffles).
__device__ __forceinline__ int gallop_search(const int* B, int lo, int nb, int x, int lane) {
    const long long off = (long long)lo + (1ll << lane) - 1;
    const int pv = (lane < 31 && off < nb) ? B[off] : INT_MAX;
    int pos = 0;  // probes below x
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int q = __shfl_sync(kFull, pv, pos + step - 1);
        if (q < x) pos += step;
    }
    int l = pos == 0 ? lo : (int)min((long long)nb, (long long)lo + (1ll << (pos - 1)));
    int h = pos >= 31 ? nb : (int)min((long long)nb, (long long)lo + (1ll << pos) - 1);
    while (l < h) {
        const int m = (l + h) >> 1;
        if (B[m] < x) l = m + 1;
        else h = m;
    }
    return l;
}

// A ∩ B written sorted to out; returns its size.
__device__ int isect_store(const int* A, int na, const int* B, int nb, int* out, int lane) {
    if (na > nb) {
        const int* t = A; A = B; B = t;
        int u = na; na = nb; nb = u;
    }
    if (prefer_merge(na, nb))
        return c_merge_vec ? warp_merge4<true>(A, na, B, nb, out, nullptr, 0, lane)
                           : warp_merge<true>(A, na, B, nb, out, nullptr, 0, lane);
    int written = 0, lo = 0;
    for (int base = 0; base < na; base += 32) {
        const int i = base + lane;
        const bool valid = i < na;
        const int x = valid ? A[i] : INT_MAX;
        const int l = gallop_search(B, lo, nb, x, lane);
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
    if (prefer_merge(na, nb))
        return c_merge_vec ? warp_merge4<false>(A, na, B, nb, nullptr, chosen, nch, lane)
                           : warp_merge<false>(A, na, B, nb, nullptr, chosen, nch, lane);
    int cnt = 0, lo = 0;
    for (int base = 0; base < na; base += 32) {
        const int i = base + lane;
        const bool valid = i < na;
        const int x = valid ? A[i] : INT_MAX;
        const int l = gallop_search(B, lo, nb, x, lane);
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
        unsigned long long old = __ldcg(&T[slot]);
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
        const unsigned long long w = __ldcg(&T[slot]);  // written by L2 atomics: skip L1
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
    int* stage;      // 2 * stage_stride(stage_cap) ints of this warp's shared memory
    int stage_cap;
    int tma;         // 1: stage fixed sets with bulk copies
    int pair_on;
    unsigned long long* ptab;  // this warp's pair-sum table (pmask + 1 words)
    unsigned long long* ptab_base;  // every warp's tables, 2^pair_log2 words each
    int pair_log2;
    unsigned pmask;
    DonationArea* don;         // null: no donation
    int split_min;             // smallest loop that is donated
    unsigned* dense;           // pool of per-vertex counter arrays for big pair sums (null: none)
    unsigned* dense_lock;      // one try-lock word per array
    int dense_slots;
    int dense_words;           // counters per array (>= v_cnt of every graph)
    unsigned* bm;              // this warp's two bitmaps over vertex ids (null: none)
    int bm_words;              // words per bitmap
    int bm_min;                // smallest fixed set tested through a bitmap
    int pair_idx;              // pair whose work is running
    long long gw;              // global warp index
    long long spw;             // ints of scratch per warp (warp w's region: scratch + (w - gw) * spw)
    unsigned long long bytes;

    // Bitmap variant of a membership test: marks set S[0, n) in bitmap r.
    // Used for fixed sets too large for shared memory when the elements to
    // test outnumber the set twice over, so the two passes over the set
    // (mark, clear) are paid back: one load per test instead of a binary
    // search of log2(n) dependent loads.  bitmap_clear undoes it.
    __device__ const unsigned* bitmap_set(const int* S, int n, int r) {
        unsigned* b = bm + (size_t)r * bm_words;
        for (int i = lane; i < n; i += 32) {
            const int x = S[i];
            atomicOr(&b[x >> 5], 1u << (x & 31));
        }
        __syncwarp();
        return b;
    }
    __device__ void bitmap_clear(const int* S, int n, int r) {
        unsigned* b = bm + (size_t)r * bm_words;
        __syncwarp();
        for (int i = lane; i < n; i += 32) b[S[i] >> 5] = 0u;
        __syncwarp();
    }
    __device__ __forceinline__ bool use_bitmap(int n, long long tests) const {
        return bm != nullptr && bm_min > 0 && n > stage_cap && n >= bm_min && tests >= 2ll * n;
    }

    // Copies a fixed set into shared-memory region r when it fits.  With
    // tma on, one lane issues a 1-D bulk copy (cp.async.bulk, completion
    // counted on the warp's mbarrier) of the 16-byte aligned span around the
    // set — the set's start rounded down, its end rounded up — and every lane
    // waits on the mbarrier; the set starts `off` ints into the region.  Set
    // sources (the CSR and the per-warp scratch) carry 16 bytes of slack past
    // their end for that round-up.
    __device__ const int* stage_set(const int* p, int n, int r) {
        if (n > stage_cap || n <= 0) return p;
        int* dst = stage + r * stage_stride(stage_cap);
#ifndef GPM_EMU
        if (tma) {
            const unsigned long long src = (unsigned long long)p;
            const unsigned long long a0 = src & ~15ull;
            const unsigned bytes = (unsigned)(((src + 4ull * (unsigned long long)n - a0) + 15ull) & ~15ull);
            const unsigned bar = (unsigned)__cvta_generic_to_shared(&s->mbar);
            const unsigned sdst = (unsigned)__cvta_generic_to_shared(dst);
            __syncwarp();  // every lane's earlier reads of the region come first
            if (lane == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                             : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        sdst),
                    "l"(a0), "r"(bytes), "r"(bar)
                    : "memory");
            }
            const unsigned ph = s->mphase;
            unsigned done = 0;
            for (int it = 0; it < (1 << 22) && !done; ++it)
                asm volatile(
                    "{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2; selp.u32 %0, 1, 0, q; }"
                    : "=r"(done)
                    : "r"(bar), "r"(ph)
                    : "memory");
            if (!__all_sync(kFull, done)) {
                if (lane == 0) record_check(kErrStage, n, (long long)src, bytes, 0, 0, 0);
            }
            __syncwarp();
            if (lane == 0) s->mphase = ph ^ 1u;
            __syncwarp();
            return dst + (int)((src - a0) >> 2);
        }
#endif
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

    // The two sides of the pair sum of level L-1 (whose loop list is set):
    // the level L-1 candidates A, the level L candidates B (below their
    // bound; neither depends on v_{L-1}) and the tail's bound.
    __device__ void pair_sides(const int*& candA, int& na, const int*& candB, int& nb, int& bnd) {
        const int L1 = P->L - 1;
        candA = s->lp[L1];
        na = s->end[L1];
        const int sb = P->loop_set[P->L];
        candB = s->ptr[sb];
        nb = lower_bound_u(candB, s->len[sb], bound_of(P->L));
        bnd = bound_of(P->T);
    }

    // Pair sums run over the two candidate lists of pair_sides, A (level
    // L-1) and B (level L), with every candidate's list length below the
    // tail bound (0 for a candidate chosen before L-1): len[j] for each
    // candidate and, per block of 32 candidates, the inclusive prefix sum of
    // the block totals.  Those arrays live in the owner's scratch: the
    // lengths in its two temporary slots (unused by pair plans, which have
    // no inclusion–exclusion tail), the block sums at the end of its region.
    // A phase then covers a flat range of list elements, so a slice is a
    // bounded number of elements wherever the hubs among the candidates sit.
    struct PairCtx {
        const int* candA;
        const int* candB;
        int na, nb, bnd;
        unsigned* lenA;
        unsigned* lenB;
        unsigned* bsA;
        unsigned* bsB;
        unsigned long long* T;  // table phases: the owner's hash table
        unsigned* cnt;          // dense phases: the owner's counter array
        unsigned ep;            // the table's tag
    };

    __device__ void pair_ctx(PairCtx& c, long long owner_w) {
        pair_sides(c.candA, c.na, c.candB, c.nb, c.bnd);
        int* base = scratch + (owner_w - gw) * spw;
        c.lenA = reinterpret_cast<unsigned*>(base + (size_t)(P->nslots - 2) * cap);
        c.lenB = reinterpret_cast<unsigned*>(base + (size_t)(P->nslots - 1) * cap);
        const long long S = pair_bs_stride(cap);
        c.bsA = reinterpret_cast<unsigned*>(base + spw - 2 * S);
        c.bsB = reinterpret_cast<unsigned*>(base + spw - S);
        c.T = nullptr;
        c.cnt = nullptr;
        c.ep = 0;
    }

    // Length units [lo, hi): blocks of 32 candidates, side A's blocks first.
    // Writes each candidate's length and each block's total.
    __device__ void pair_length_blocks(const PairCtx& c, int lo, int hi) {
        const int L1 = P->L - 1;
        const int nba = (c.na + 31) >> 5;
        for (int u = lo; u < hi; ++u) {
            const bool sa = u < nba;
            const int b = sa ? u : u - nba;
            const int* cand = sa ? c.candA : c.candB;
            const int n = sa ? c.na : c.nb;
            unsigned* len = sa ? c.lenA : c.lenB;
            unsigned* bs = sa ? c.bsA : c.bsB;
            const int j = (b << 5) + lane;
            int l = 0;
            if (j < n) {
                const int v = cand[j];
                if (!chosen_before(v, L1)) {
                    const unsigned st = g.rowptr[v];
                    l = lower_bound_u(g.col + st, (int)(g.rowptr[v + 1] - st), c.bnd);
                }
                len[j] = (unsigned)l;
            }
            int pre;
            const int tot = warp_scan(l, pre);
            if (lane == 0) bs[b] = (unsigned)tot;
        }
        __syncwarp();
    }

    // bs[0, nblk) <- inclusive prefix sums in place; returns the total (the
    // candidates are distinct vertices, so it is below the edge count < 2^32)
    __device__ unsigned pair_scan(unsigned* bs, int nblk) {
        unsigned carry = 0;
        for (int base = 0; base < nblk; base += 32) {
            const int b = base + lane;
            unsigned incl = b < nblk ? __ldcg(&bs[b]) : 0u;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned t = __shfl_up_sync(kFull, incl, o);
                if (lane >= o) incl += t;
            }
            if (b < nblk) bs[b] = carry + incl;
            carry += __shfl_sync(kFull, incl, 31);
        }
        __syncwarp();
        return carry;
    }

    // The block holding element e0: the number of blocks whose inclusive sum
    // is at most e0 (a 32-way search: each step probes 32 evenly spaced
    // blocks and keeps the gap where the sums pass e0).
    __device__ int pair_first_block(const unsigned* bs, int nblk, unsigned long long e0) const {
        int lo = 0, hi = nblk;  // the answer is in [lo, hi]
        while (hi - lo > 32) {
            const int step = (hi - lo + 31) >> 5;
            const int p = lo + (lane + 1) * step - 1;
            const bool le = p < hi && (unsigned long long)__ldcg(&bs[p]) <= e0;
            const int c = __popc(__ballot_sync(kFull, le));
            const int pc = lo + (c + 1) * step - 1;  // first probe above e0, if any
            if (pc < hi) hi = pc;
            lo += c * step;
        }
        const bool le = lo + lane < hi && (unsigned long long)__ldcg(&bs[lo + lane]) <= e0;
        return lo + __popc(__ballot_sync(kFull, le));
    }

    // Elements [e0, e1) of one side's concatenated neighbour lists (below
    // the bound), each x not chosen before L-1: phase 0 adds one to x's
    // count, phase 1 sums the counts (this lane's share), phase 2 zeroes
    // them.  Counts live in the table T (tag ep) or, when cnt is set, in the
    // dense array cnt indexed by vertex.  In phase 1 a candidate w that is on
    // the other side too (`other`) pairs with itself once per element:
    // those are the v == w terms of sum_x a_x b_x, subtracted here.
    __device__ long long pair_flat(const int* cand, int n, const unsigned* len, const unsigned* bs, const int* other,
                                   int nother, unsigned long long* T, unsigned* cnt, unsigned ep, int phase,
                                   unsigned long long e0, unsigned long long e1) {
        const int L1 = P->L - 1;
        const int nblk = (n + 31) >> 5;
        long long sum = 0;
        for (int b = pair_first_block(bs, nblk, e0); b < nblk; ++b) {
            const unsigned long long b0 = b ? (unsigned long long)__ldcg(&bs[b - 1]) : 0ull;
            if (b0 >= e1) break;
            const int j = (b << 5) + lane;
            const int l = j < n ? (int)__ldcg(&len[j]) : 0;
            int pre;
            warp_scan(l, pre);
            const unsigned long long s0 = b0 + (unsigned)pre, s1 = s0 + (unsigned)l;
            const unsigned long long a = s0 > e0 ? s0 : e0, z = s1 < e1 ? s1 : e1;
            int m = 0;
            unsigned st = 0;
            int dup = 0;
            if (a < z) {
                m = (int)(z - a);
                const int v = cand[j];
                st = g.rowptr[v] + (unsigned)(a - s0);
                if (phase == 1) dup = contains(other, nother, v) ? 1 : 0;
                if (kBytes) bytes += 4ull * (unsigned long long)m + 8;
            }
            int pm;
            const int M = warp_scan(m, pm);
            for (int eb = 0; eb < M; eb += 32) {
                const int e = eb + lane;
                const int c = owner(pm, e);
                const unsigned stc = __shfl_sync(kFull, st, c);
                const int pc = __shfl_sync(kFull, pm, c);
                const int dc = __shfl_sync(kFull, dup, c);
                if (e < M) {
                    const int x = g.col[stc + (e - pc)];
                    if (!chosen_before(x, L1)) {
                        if (cnt) {
                            if (phase == 0) atomicAdd(&cnt[x], 1u);
                            else if (phase == 1) sum += (long long)__ldcg(&cnt[x]) - dc;
                            else cnt[x] = 0u;
                        } else if (phase == 0) {
                            if (!pair_add(T, pmask, ep, x)) record_check(3, x, n, pmask, 0, 0, 0);
                        } else {
                            sum += (long long)pair_get(T, pmask, ep, x) - dc;
                        }
                    }
                }
            }
            __syncwarp();
        }
        return sum;
    }

    // One slice [lo, hi) of a pair-sum phase; returns this lane's share of
    // the probe sums.  Element phases count units of 2^(kind >> 16) elements.
    __device__ long long pair_run(const PairCtx& c, int kind, int lo, int hi) {
        if ((kind & 0xff) == kDonPairLen) {
            pair_length_blocks(c, lo, hi);
            return 0;
        }
        const bool sa = (kind & kDonSideA) != 0;
        const int ul = (kind >> 16) & 31;
        return pair_flat(sa ? c.candA : c.candB, sa ? c.na : c.nb, sa ? c.lenA : c.lenB, sa ? c.bsA : c.bsB,
                         sa ? c.candB : c.candA, sa ? c.nb : c.na, c.T, c.cnt, c.ep, don_phase(kind),
                         (unsigned long long)lo << ul, (unsigned long long)hi << ul);
    }

    // Publishes one phase of a shared pair sum in slot h (held by this
    // warp): `units` units, a new generation; tag is the table's epoch or
    // the dense array's index, aux the side's candidate count (the length
    // phase: side A's).  Returns the generation (on every lane).
    __device__ unsigned pair_publish(int h, int kind, int units, unsigned tag, int aux) {
        unsigned gen = 0;
        __syncwarp();
        if (lane == 0) {
            Donation* r = &don->rec[h];
            volatile Donation* vr = r;
            gen = ((unsigned)(vr->word >> 48) + 1u) & 0xffffu;
            vr->pair = pair_idx;
            vr->depth = P->L - 1;
            vr->kind = kind;
            vr->owner = (int)gw;
            vr->epoch = tag;
            vr->done = 0u;
            for (int j = 0; j < P->L - 1; ++j) vr->chosen[j] = s->chosen[j];
            vr->chosen[kMaxN - 1] = aux;
            __threadfence();
            atomicExch(&r->word, don_pack(gen, (unsigned)units, 0u));
        }
        return __shfl_sync(kFull, gen, 0);
    }

    // Takes slices of one pair-sum phase (record h, generation gen) until
    // none is left; every finished slice is added to the record's done
    // count.  Returns this lane's share of the probe sums.
    __device__ long long pair_slices(int h, unsigned gen, int kind, const PairCtx& c) {
        Donation* r = &don->rec[h];
        long long sum = 0;
        for (;;) {
            int lo = 0, hi = 0;
            if (lane == 0) don_claim(r, gen, kind, lo, hi);
            lo = __shfl_sync(kFull, lo, 0);
            hi = __shfl_sync(kFull, hi, 0);
            if (hi <= lo) break;
            sum += pair_run(c, kind, lo, hi);
            __syncwarp();
            if (lane == 0) {
                __threadfence();  // the slice's writes before its count
                atomicAdd(&r->done, (unsigned)(hi - lo));
            }
        }
        return sum;
    }

    // Waits until every slice of the phase in record h is finished (the
    // helpers holding slices are running, so the wait ends); bounded, and
    // recorded as a check failure if the bound is reached.
    __device__ bool pair_wait(int h, int n) {
        unsigned d = 0;
        for (int it = 0; it < (1 << 24); ++it) {
            if (lane == 0) d = atomicAdd(&don->rec[h].done, 0u);
            d = __shfl_sync(kFull, d, 0);
            if (d >= (unsigned)n) {
                __threadfence();
                return true;
            }
            __nanosleep(256);
        }
        if (lane == 0) record_check(kErrDonation, h, n, d, 0, 0, 2);
        return false;
    }

    // A free donation slot for this warp, or -1 (lane 0 searches).
    __device__ int take_slot(int salt) {
        int h = -1;
        if (lane == 0) {
            h = don_take_slot(don, gw * 7 + salt * 131);
            if (h >= 0) atomicAdd(&don->held, 1u);
        }
        return __shfl_sync(kFull, h, 0);
    }

    // Before this owner publishes another phase in record h: every helper of
    // the last phase has left (they leave once it is exhausted); bounded.
    __device__ void pair_vacate(int h) {
        unsigned v = 0;
        for (int it = 0; it < (1 << 24); ++it) {
            if (lane == 0) v = atomicAdd(&don->visits[h], 0u);
            v = __shfl_sync(kFull, v, 0);
            if (v == 0) return;
            __nanosleep(128);
        }
        if (lane == 0) record_check(kErrDonation, h, v, 0, 0, 0, 6);
    }

    __device__ void drop_slot(int h) {
        if (h < 0) return;
        __syncwarp();
        if (lane == 0) {
            __threadfence();
            atomicExch(&don->busy[h], 0u);
            atomicAdd(&don->held, ~0u);  // minus one
        }
        __syncwarp();
    }

    // One phase over all of its units: shared through slot h, or by this
    // warp alone when h < 0.
    __device__ long long pair_phase(const PairCtx& c, int h, int kind, int units, unsigned tag, int aux) {
        if (h < 0) return pair_run(c, kind, 0, units);
        pair_vacate(h);
        const unsigned gen = pair_publish(h, kind, units, tag, aux);
        const long long sum = pair_slices(h, gen, kind, c);
        pair_wait(h, units);
        return sum;
    }

    // Sum over (v, w), v a level L-1 candidate, w a level L candidate, v != w,
    // of |N(v) ∩ N(w) ∩ [0, bound) \ chosen|, as sum_x a_x b_x - c (the
    // plan's pair_ok shape; c the v == w terms).  Level L-1's loop list is
    // set.  The smaller side (by list elements) counts its neighbours into
    // this warp's hash table when it fills it at most half, else into a
    // dense per-vertex counter array from the pool (zeroed again after);
    // the other side sums the counts.  Long pair sums are shared with idle
    // warps phase by phase (lengths, count, sum, zero).  Returns false (and
    // counts nothing) when a dense array is needed and none is free, or the
    // work is too long for one warp and no donation slot is free: the
    // caller then runs the level normally.
    __device__ bool pair_level(__int128& out) {
        constexpr long long kDenseMaxOps = 1ll << 24;  // one warp's longest dense pair sum
        constexpr int kShareBlocks = GPM_PAIR_SHARE_BLOCKS;
        const int L1 = P->L - 1;
        PairCtx c;
        pair_ctx(c, gw);
        out = 0;
        if (c.na == 0 || c.nb == 0) return true;
        const int nba = (c.na + 31) >> 5, nbb = (c.nb + 31) >> 5;
        const bool can_share = don && split_min > 0 && nba + nbb <= (int)kDonEndMax;
        int h = (can_share && nba + nbb >= kShareBlocks) ? take_slot(L1) : -1;
        pair_phase(c, h, kDonPairLen, nba + nbb, 0u, c.na);
        const unsigned ma = pair_scan(c.bsA, nba), mb = pair_scan(c.bsB, nbb);
        if (ma == 0 || mb == 0) {
            drop_slot(h);
            return true;
        }
        const unsigned long long total = (unsigned long long)ma + mb;
        if (c_pair_max_ops > 0 && (long long)total > c_pair_max_ops) {
            drop_slot(h);
            return false;
        }
        if (h < 0 && can_share && total >= 64ull * (unsigned long long)split_min) h = take_slot(L1);
        const bool a_fills = ma < mb;
        const unsigned mins = a_fills ? ma : mb, maxs = a_fills ? mb : ma;
        int dslot = -1;
        unsigned tag;
        if (2ull * mins > (unsigned long long)pmask + 1ull) {
            // too big for the table: a dense counter array
            if (!dense || g.v_cnt > dense_words || (h < 0 && (long long)(total + mins) > kDenseMaxOps)) {
                drop_slot(h);
                return false;
            }
            if (lane == 0) {
                for (int i = 0; i < dense_slots && dslot < 0; ++i) {
                    const int k = (int)((gw + i) % dense_slots);
                    if (atomicCAS(&dense_lock[k], 0u, 1u) == 0u) dslot = k;
                }
            }
            dslot = __shfl_sync(kFull, dslot, 0);
            if (dslot < 0) {
                drop_slot(h);
                return false;
            }
            c.cnt = dense + (size_t)dslot * (size_t)dense_words;
            tag = (unsigned)dslot;
        } else {
            __syncwarp();
            if (lane == 0) {
                s->epoch = (s->epoch + 1) & 0xffffu;
                if (s->epoch == 0) s->epoch = 1;
            }
            __syncwarp();
            c.ep = s->epoch;
            c.T = ptab;
            if (c.ep == 1) {  // fresh cycle of tags: clear the table
                for (unsigned i = lane; i <= pmask; i += 32) ptab[i] = 0ull;
                __syncwarp();
            }
            tag = c.ep;
        }
        // element units: 2^GPM_PAIR_UNIT_LOG2 elements, coarser when a side
        // would exceed 2^24 units
        int ul = GPM_PAIR_UNIT_LOG2;
        while (((unsigned long long)maxs >> ul) >= (unsigned long long)kDonEndMax) ++ul;
        const unsigned long long um = (1ull << ul) - 1;
        const int ufill = (int)((mins + um) >> ul), uprobe = (int)((maxs + um) >> ul);
        const int fside = a_fills ? kDonSideA : 0, pside = a_fills ? 0 : kDonSideA;
        const int nfill = a_fills ? c.na : c.nb, nprobe = a_fills ? c.nb : c.na;
        const int kf = c.cnt ? kDonDenseFill : kDonPairFill, kp = c.cnt ? kDonDenseProbe : kDonPairProbe;
        long long sum = 0;
        pair_phase(c, h, kf | fside | (ul << 16), ufill, tag, nfill);
        sum += pair_phase(c, h, kp | pside | (ul << 16), uprobe, tag, nprobe);
        if (c.cnt) pair_phase(c, h, kDonDenseClear | fside | (ul << 16), ufill, tag, nfill);
        drop_slot(h);
        if (dslot >= 0) {
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                atomicExch(&dense_lock[dslot], 0u);
            }
            __syncwarp();
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
        out = lane == 0 ? (__int128)sum : (__int128)0;
        return true;
    }

    // Σ deg(v) over the candidates not chosen before depth L (warp-uniform)
    __device__ long long list_total(const int* cand, int ncand, int L) {
        long long m = 0;
        for (int base = 0; base < ncand; base += 32) {
            const int j = base + lane;
            int len = 0;
            if (j < ncand) {
                const int v = cand[j];
                if (!chosen_before(v, L)) len = (int)(g.rowptr[v + 1] - g.rowptr[v]);
            }
            int pre;
            m += warp_scan(len, pre);
        }
        return m;
    }

    // Candidates [lo, hi) of level L at once (the plan's leaf_kind says how
    // the tail reads N(v)); chosen[0, L) and the level's loop list are set.
    // The result is a sum over candidates, so slices add up.
    __device__ __int128 leaf_batch(int lo, int hi) {
        const int L = P->L, T = P->T;
        const int* cand = s->lp[L] + lo;
        const int ncand = hi - lo;
        long long total = 0;
        if (P->leaf_kind == kLeafCount) {
            // bound of the last loop: restrictions on depths < L are fixed
            const unsigned m = P->rmask[T];
            int bfix = g.v_cnt;
            for (int j = 0; j < L; ++j)
                if (m >> j & 1) bfix = min(bfix, s->chosen[j]);
            const bool by_v = (m >> L) & 1;
            const int* F = nullptr;
            const unsigned* FB = nullptr;
            int nf = 0, lim = bfix;
            if (P->leaf_fa >= 0) {
                nf = lower_bound_u(s->ptr[P->leaf_fa], s->len[P->leaf_fa], bfix);
                if (nf == 0) return 0;
                F = stage_set(s->ptr[P->leaf_fa], nf, 0);
                lim = min(bfix, F[nf - 1] + 1);
                if (use_bitmap(nf, list_total(cand, ncand, L))) FB = bitmap_set(F, nf, 0);
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
                        if (hit && F) hit = FB ? ((FB[x >> 5] >> (x & 31)) & 1u) != 0 : contains(F, nf, x);
                    }
                    total += __popc(__ballot_sync(kFull, hit));
                }
            }
            if (FB) bitmap_clear(F, nf, 0);
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
        const unsigned* BA = nullptr;
        const unsigned* BB = nullptr;
        if (bm && ((Pa && na > stage_cap) || (Pb && nb > stage_cap))) {
            const long long tests = both_fixed ? (long long)ncand : list_total(cand, ncand, L);
            if (Pa && use_bitmap(na, tests)) BA = bitmap_set(Pa, na, 0);
            if (Pb && Pb == Pa) BB = BA;
            else if (Pb && use_bitmap(nb, tests)) BB = bitmap_set(Pb, nb, 1);
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
                if (ka == 0) inA = BA ? ((BA[v >> 5] >> (v & 31)) & 1u) != 0 : contains(Pa, na, v);
                if (kb == 0) inB = BB ? ((BB[v >> 5] >> (v & 31)) & 1u) != 0 : contains(Pb, nb, v);
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
                        ma = ka == 1 ? true : (BA ? ((BA[x >> 5] >> (x & 31)) & 1u) != 0 : contains(Pa, na, x));
                        mb = kb == 1 ? true : (BB ? ((BB[x >> 5] >> (x & 31)) & 1u) != 0 : contains(Pb, nb, x));
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
        if (BA) bitmap_clear(Pa, na, 0);
        if (BB && BB != BA) bitmap_clear(Pb, nb, 1);
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) total += __shfl_xor_sync(kFull, total, o);
        return lane == 0 ? (__int128)total : (__int128)0;
    }

    // N(v); an id outside the graph is recorded and reads as isolated
    __device__ __forceinline__ void nbr(int v, const int*& p, int& d) const {
        if ((unsigned)v >= (unsigned)g.v_cnt) {
            if (lane == 0) record_check(kErrBadVertex, v, g.v_cnt, P->n, 0, 0, 0);
            p = g.col;
            d = 0;
            return;
        }
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

    // Lane 0 writes warp-shared state only between two __syncwarp: the first
    // orders the other lanes' earlier reads before the write (no lane may
    // see the new value early), the second publishes it.
    __device__ __forceinline__ void set_chosen(int d, int v) {
        __syncwarp();
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
                if (min(lf, dv) > cap) {  // an intersection larger than its slot
                    if (lane == 0) record_check(kErrSetSize, pid, lf, dv, cap, 0, 0);
                    return false;
                }
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
        __syncwarp();
        if (lane == 0) {
            s->lp[d] = S;
            s->idx[d] = 0;
            s->end[d] = e;
            s->dslot[d] = -1;
        }
        __syncwarp();
    }

    // Publishes the loop of depth d (just started) when it is long enough —
    // split_min candidates, or fewer whose neighbour lists hold at least
    // kLoopBudget elements (a short loop over hubs: each iteration is a
    // long intersection) — and a slot is free; the owner's own range then
    // comes from claims.
    __device__ void maybe_donate(int d) {
        if (!don || split_min <= 0) return;
        const int e = s->end[d];
        if (e < 2 || e > (int)kDonEndMax) return;
        if (e < split_min) {
            const int* list = s->lp[d];
            unsigned long long work = 0;
            for (int base = 0; base < e; base += 32) {
                const int j = base + lane;
                unsigned dg = 0;
                if (j < e) {
                    const int v = list[j];
                    dg = g.rowptr[v + 1] - g.rowptr[v];
                }
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) dg += __shfl_xor_sync(kFull, dg, o);
                work += dg;
            }
            if (work < kLoopBudget) return;
        }
        __syncwarp();
        if (lane == 0) {
            const int h = don_take_slot(don, gw * 7 + d * 131);
            if (h >= 0) {
                atomicAdd(&don->held, 1u);
                Donation* r = &don->rec[h];
                volatile Donation* vr = r;
                const unsigned gen = ((unsigned)(vr->word >> 48) + 1u) & 0xffffu;
                vr->pair = pair_idx;
                vr->depth = d;
                vr->kind = (d == P->L && batch_on()) ? kDonLeaf : kDonLoop;
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

    // Next slice of the donated loop at depth d into idx[d], end[d].  A loop
    // slice is weighted: its candidates' neighbour lists (their degrees, the
    // cost of the intersections below them) add up to at most kLoopBudget
    // elements, or it is one candidate.  Loop lists run in id order, which is
    // descending degree, so the hubs at a loop's start come one per slice
    // instead of 64 to the first claimer.
    __device__ bool claim_more(int d) {
        __syncwarp();
        if ((unsigned)s->dslot[d] >= (unsigned)kDonSlots) {
            if (lane == 0) record_check(kErrDonation, d, s->dslot[d], 0, 0, 0, 1);
            return false;
        }
        Donation* r = &don->rec[s->dslot[d]];
        const unsigned gen = s->dgen[d] & 0xffffu;
        const bool leaf = d == P->L && batch_on();
        const int* list = s->lp[d];
        int lo = 0, hi = 0;
        unsigned long long w = 0;
        if (lane == 0) w = *(volatile unsigned long long*)&r->word;
        w = __shfl_sync(kFull, w, 0);
        const unsigned end = (unsigned)(w >> 24) & 0xffffffu, next = (unsigned)w & 0xffffffu;
        if ((unsigned)(w >> 48) == gen && next < end) {
            const unsigned smin = leaf ? 8u : 1u, smax = leaf ? 128u : 64u;
            unsigned take = min(end - next, min(smax, max(smin, (end - next) >> 5)));
            if (!leaf) {
                // weighted from the candidates at the snapshot's next: the
                // add may land further on, where degrees are no larger
                const unsigned look = min(take, 32u);
                unsigned dg = 0;
                if ((unsigned)lane < look) {
                    const int v = list[next + lane];
                    dg = g.rowptr[v + 1] - g.rowptr[v];
                }
                unsigned incl = dg;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const unsigned t = __shfl_up_sync(kFull, incl, o);
                    if (lane >= o) incl += t;
                }
                const unsigned fit = __popc(__ballot_sync(kFull, (unsigned)lane < look && incl <= kLoopBudget));
                if (fit < look) take = max(1u, fit);
            }
            if (lane == 0) don_take(r, gen, take, lo, hi);
            lo = __shfl_sync(kFull, lo, 0);
            hi = __shfl_sync(kFull, hi, 0);
        }
        __syncwarp();
        if (lane == 0 && hi > lo) {
            s->idx[d] = lo;
            s->end[d] = hi;
        }
        __syncwarp();
        return hi > lo;
    }

    // the donated loop at depth d is exhausted: its owner frees the slot, a
    // helper ends its visit
    __device__ void release(int d) {
        __syncwarp();
        if (lane == 0) {
            if ((unsigned)s->dslot[d] < (unsigned)kDonSlots) {
                if (s->downer[d]) {
                    __threadfence();
                    atomicExch(&don->busy[s->dslot[d]], 0u);
                    atomicAdd(&don->held, ~0u);  // minus one
                } else {
                    don_leave(don, s->dslot[d]);
                }
            }
            s->dslot[d] = -1;
        }
        __syncwarp();
    }

    __device__ __forceinline__ bool batch_on() const { return leaf_on && P->leaf_kind != kLeafGeneric; }
    // pair-sum table keys are 24-bit ids
    __device__ __forceinline__ bool pair_ready() const { return pair_on && P->pair_ok && g.v_cnt <= (1 << 24); }

    // The batched deepest level: its range [idx, end), then (when the level
    // is published) every further slice the warp can claim.
    __device__ __int128 leaf_slices() {
        const int L = P->L;
        __int128 acc = 0;
        for (;;) {
            const int lo = s->idx[L], hi = s->end[L];
            if (lo < hi) acc += leaf_batch(lo, hi);
            if (s->dslot[L] < 0) break;
            if (!claim_more(L)) {
                release(L);
                break;
            }
        }
        return acc;
    }

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
            if (i >= s->len[P->loop_set[d]]) {  // a loop range beyond its set
                if (lane == 0) record_check(kErrLoopIndex, d, i, s->end[d], s->len[P->loop_set[d]], s->dslot[d], 0);
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
                maybe_donate(L);
                acc += leaf_slices();
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
        if (batch_on() && L == 2) {
            maybe_donate(2);
            return leaf_slices();
        }
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
        int lo = 0, hi = 0, p = 0, d = 0, rend = 0, kind = 0, owner_w = 0, aux = 0;
        unsigned ep = 0;
        if (lane == 0) {
            // a visitor from here on: no new generation is published in r
            // until it leaves, so the fields read below stay the record's
            don_visit(don, h);
            const unsigned long long w = *(volatile unsigned long long*)&r->word;
            if ((unsigned)(w >> 48) == gen && (w & 0xffffffu) < ((w >> 24) & 0xffffffu)) {
                __threadfence();
                const volatile Donation* vr = r;
                p = vr->pair;
                d = vr->depth;
                for (int j = 0; j < kMaxN; ++j) s->chosen[j] = j < d ? vr->chosen[j] : -1;
                kind = vr->kind;
                owner_w = vr->owner;
                ep = vr->epoch;
                aux = vr->chosen[kMaxN - 1];
                rend = (int)((w >> 24) & 0xffffffu);
                don_claim(r, gen, kind, lo, hi);
            }
            if (hi <= lo) don_leave(don, h);
        }
        lo = __shfl_sync(kFull, lo, 0);
        hi = __shfl_sync(kFull, hi, 0);
        p = __shfl_sync(kFull, p, 0);
        d = __shfl_sync(kFull, d, 0);
        rend = __shfl_sync(kFull, rend, 0);
        kind = __shfl_sync(kFull, kind, 0);
        owner_w = __shfl_sync(kFull, owner_w, 0);
        ep = __shfl_sync(kFull, ep, 0);
        aux = __shfl_sync(kFull, aux, 0);
        __syncwarp();
        if (hi <= lo) return false;
        const bool pair_kind = don_pair_kind(kind);
        const bool dense_kind = don_dense_kind(kind);
        const bool len_kind = (kind & 0xff) == kDonPairLen;
        // pair sums: the owner's warp index locates its arrays (and table);
        // a dense phase's tag is its counter array
        const bool bad_owner =
            pair_kind && ((unsigned)owner_w >= gridDim.x * (blockDim.x >> 5) ||
                          (dense_kind ? (!dense || ep >= (unsigned)dense_slots) : (!len_kind && !ptab_base)));
        if (p < 0 || p >= npairs || bad_owner) {
            if (lane == 0) {
                record_check(kErrDonation, h, p, d, lo, hi, rend);
                don_leave(don, h);
            }
            __syncwarp();
            return true;
        }
        const PairDesc pd = pairs[p];
        P = pd.plan;
        g = pd.g;
        cap = pd.cap;
        pair_idx = p;
        bool ok = d >= 2 && d <= P->L && (!pair_kind || (d == P->L - 1 && P->pair_ok));
        for (int l = 0; l < d && ok; ++l) {
            const int* nv;
            int dv;
            nbr(s->chosen[l], nv, dv);
            ok = build_chain(l, nv, dv);
        }
        if (ok) start_level(d);
        PairCtx pc;
        if (ok && pair_kind) {
            // the owner's pair sum as this warp rebuilds it: the same lists
            pair_ctx(pc, owner_w);
            if (len_kind) ok = aux == pc.na && rend == ((pc.na + 31) >> 5) + ((pc.nb + 31) >> 5);
            else ok = aux == ((kind & kDonSideA) ? pc.na : pc.nb);
        } else if (ok) {
            ok = s->end[d] == rend;
        }
        if (!ok) {
            // the rebuilt loop differs from the published one: the slice is lost
            if (lane == 0) {
                record_check(kErrDonation, h, p, d, lo, hi, rend);
                don_leave(don, h);
            }
            __syncwarp();
            return true;
        }
        if (pair_kind) {
            if (dense_kind) {
                if (g.v_cnt > dense_words) {
                    if (lane == 0) {
                        record_check(kErrDonation, h, p, d, lo, hi, -3);
                        don_leave(don, h);
                    }
                    __syncwarp();
                    return true;
                }
                pc.cnt = dense + (size_t)ep * (size_t)dense_words;
            } else if (!len_kind) {
                pc.T = ptab_base + ((size_t)owner_w << pair_log2);
                pc.ep = ep;
            }
            long long sum = pair_run(pc, kind, lo, hi);
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                atomicAdd(&r->done, (unsigned)(hi - lo));
            }
            sum += pair_slices(h, gen, kind, pc);
            __syncwarp();
            if (lane == 0) don_leave(don, h);  // the phase is exhausted
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) sum += __shfl_xor_sync(kFull, sum, o);
            if (lane == 0 && sum != 0) add128(out + 2 * p, (__int128)sum);
            return true;
        }
        __syncwarp();  // every lane has read end[d] above
        if (lane == 0) {
            s->idx[d] = lo;
            s->end[d] = hi;
            s->dslot[d] = h;
            s->dgen[d] = gen;
            s->downer[d] = 0;
        }
        __syncwarp();
        const __int128 acc = (d == P->L && batch_on()) ? leaf_slices() : dfs_levels(d);
        if (s->dslot[d] >= 0) release(d);  // left early (an internal check): end the visit
        if (lane == 0 && acc != 0) add128(out + 2 * p, acc);
        return true;
    }

    // After the warp's own queues: helps published loops until every warp
    // is done.  The host clamps the grid to the blocks that are resident at
    // once, so every other warp is running and the wait ends when they do;
    // the polling is bounded all the same (2^24 rounds of at least 4 us; a
    // helper that stops early only leaves work to the owners).  The records
    // are scanned only while some owner holds a slot.
    __device__ void help_all(const PairDesc* pairs, int npairs, unsigned long long* out, unsigned total_warps) {
        for (unsigned round = 0; round < (1u << 24); ++round) {
            bool worked = false;
            unsigned held = 0;
            if (lane == 0) held = *(volatile unsigned*)&don->held;
            held = __shfl_sync(kFull, held, 0);
            for (int base = 0; held && base < kDonSlots; base += 32) {
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
            if (worked) continue;
            // one lane reads the counter: the exit must be warp-uniform
            unsigned fin = 0;
            if (lane == 0) fin = *(volatile unsigned*)&don->finished;
            if (__shfl_sync(kFull, fin, 0) >= total_warps) return;
            __nanosleep(held ? 8000 : 4000);
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

// kMinBlocks 1: any block up to 16 warps; 3 or 4: blocks of at most 8 warps,
// three or four resident per SM (the register budget drops to 80 or 64, with
// spills to local memory); 5: blocks of at most 4 warps, five per SM (96
// registers, few spills) — more warps in flight
template <bool kBytes, int kMinBlocks>
__global__ void __launch_bounds__(kMinBlocks == 1 ? 512 : (kMinBlocks == 5 ? 128 : 256), kMinBlocks) match_kernel(const PairDesc* __restrict__ pairs, int npairs,
                                                    unsigned long long* __restrict__ cursors,
                                                    unsigned long long* __restrict__ out, int* __restrict__ scratch_all,
                                                    long long scratch_per_warp, int chunk,
                                                    const unsigned long long* __restrict__ params,
                                                    int leaf_on, int stage_cap, int pair_on,
                                                    unsigned long long* __restrict__ pair_tables, int pair_log2,
                                                    DonationArea* don, int split_min, unsigned* bitmaps,
                                                    int bm_words, int bm_min, unsigned* dense_pool,
                                                    int dense_slots, int dense_words,
                                                    unsigned long long* __restrict__ stats) {
    // params[0] = stripes, params[1] = stripe (device memory, so a captured
    // graph can replay with new values)
    const unsigned long long stripes = params[0], stripe = params[1];
#ifdef GPM_EMU
    unsigned char* smem_raw = gpm_emu::block_shared();
#else
    extern __shared__ __align__(16) unsigned char smem_raw[];
#endif
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const long long gw = (long long)blockIdx.x * nwarps + wid;
    WarpCtx<kBytes> w;
    w.s = reinterpret_cast<WarpState*>(smem_raw) + wid;
    w.stage = reinterpret_cast<int*>(reinterpret_cast<WarpState*>(smem_raw) + nwarps) +
              (size_t)wid * 2 * stage_stride(stage_cap);
    w.stage_cap = stage_cap;
    // leaf_on: bit 0 the batched deepest level, bit 1 bulk-copy staging
    w.leaf_on = leaf_on & 1;
    w.tma = (leaf_on >> 1) & 1;
#ifndef GPM_EMU
    if (w.tma) {
        if (lane == 0) {
            const unsigned bar = (unsigned)__cvta_generic_to_shared(&w.s->mbar);
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            w.s->mphase = 0;
        }
        __syncwarp();
    }
#endif
    w.pair_on = pair_on && pair_tables != nullptr;
    w.pmask = (1u << pair_log2) - 1u;
    w.ptab = pair_tables ? pair_tables + ((size_t)gw << pair_log2) : nullptr;
    w.ptab_base = pair_tables;
    w.pair_log2 = pair_log2;
    // Each warp's table keeps its entries across launches: the warp's last
    // tag is stored after all tables (one word per warp), so a table is
    // cleared only when its cycle of tags wraps, not in every launch.  A
    // stored 0 (tables just zeroed by the host) reads as 1, a tag no entry
    // of a zeroed table carries.
    unsigned* const pair_epochs =
        pair_tables ? reinterpret_cast<unsigned*>(pair_tables + (((size_t)gridDim.x * nwarps) << pair_log2)) : nullptr;
    if (lane == 0) {
        const unsigned e = pair_epochs ? pair_epochs[gw] : 0u;
        w.s->epoch = e ? e : 1u;
    }
    w.scratch = scratch_all + gw * scratch_per_warp;
    w.spw = scratch_per_warp;
    w.lane = lane;
    w.bytes = 0;
    w.don = don;
    w.split_min = split_min;
    w.gw = gw;
    w.dense_slots = dense_pool ? dense_slots : 0;
    w.dense_words = dense_words;
    w.dense_lock = dense_pool;  // dense_slots lock words, then 64-word aligned arrays
    w.dense = dense_pool ? dense_pool + ((dense_slots + 63) & ~63) : nullptr;
    w.bm = bitmaps ? bitmaps + (size_t)gw * 2 * (size_t)bm_words : nullptr;
    w.bm_words = bm_words;
    w.bm_min = bm_min;
    // Each warp starts at its own pair (warp index mod pairs) and then visits
    // all of them, so the heavy pairs' tasks start at once instead of after
    // every warp has worked through the pairs before them.
    const int p0 = (int)(gw % npairs);
    for (int k = 0; k < npairs; ++k) {
        const int p = p0 + k < npairs ? p0 + k : p0 + k - npairs;
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
    if (lane == 0 && pair_epochs) pair_epochs[gw] = w.s->epoch;
}
