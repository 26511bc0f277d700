// CPU warp emulator for the matcher's device core (test infrastructure).
//
// graphpi_gb300/csrc/match_core.cuh compiles as host C++ against this file:
// every warp of a launch runs on one host thread, its 32 lanes as
// cooperative contexts (ucontext) that take turns up to each warp-wide
// intrinsic (shuffle, ballot, match, __syncwarp), which acts as a barrier;
// atomics map to GCC __atomic builtins, so warps race as on the GPU.  Run
// under AddressSanitizer it checks the kernel's indexing on small graphs
// without a GPU, and a lane that returns while the others wait at an
// intrinsic (a divergent warp-wide call) stops the run.
#pragma once
#include <ucontext.h>

#include <climits>
#include <source_location>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <type_traits>
#include <vector>

#if defined(__SANITIZE_ADDRESS__)
#include <sanitizer/common_interface_defs.h>
#define GPM_EMU_ASAN 1
#endif

#define GPM_EMU 1
#define __device__
#define __global__
#define __host__
#define __forceinline__ inline
#define __noinline__ __attribute__((noinline))
#define __launch_bounds__(...)
#define __constant__
#define __shared__
#define __align__(n) alignas(n)

namespace gpm_emu {

struct Dim {
    unsigned x = 0, y = 0, z = 0;
};

struct Thread {
    Dim tid, bid;
    unsigned char* smem = nullptr;
};

// One warp = one host thread; its 32 lanes are cooperative contexts that
// run in turn until each reaches the next warp-wide intrinsic (a barrier).
struct Warp {
    ucontext_t sched;
    ucontext_t lane_ctx[32];
    std::vector<char> stacks;
    Thread th[32];
    unsigned long long slot[2][32];
    int parity[32] = {0};
    bool done[32] = {false};
    int cur = 0;
    // call site of each lane's pending intrinsic
    unsigned site[32] = {0};
    const char* site_file[32] = {nullptr};
    unsigned hist[32][16] = {{0}};  // last call-site lines per lane
    unsigned nhist[32] = {0};
    const void* sched_bottom = nullptr;
    size_t sched_size = 0;
};

inline thread_local Thread t;
inline thread_local Warp* t_warp = nullptr;
inline Dim block_dim, grid_dim;

inline unsigned char* block_shared() { return t.smem; }
inline unsigned lane() { return t.tid.x & 31u; }

// lane -> scheduler (the lane waits at a barrier)
inline void yield_lane(unsigned site = 0, const char* file = nullptr) {
    Warp* w = t_warp;
    const int l = w->cur;
    w->site[l] = site;
    w->site_file[l] = file;
    w->hist[l][w->nhist[l]++ & 15] = site;
#ifdef GPM_EMU_ASAN
    void* fake = nullptr;
    __sanitizer_start_switch_fiber(&fake, w->sched_bottom, w->sched_size);
#endif
    swapcontext(&w->lane_ctx[l], &w->sched);
#ifdef GPM_EMU_ASAN
    __sanitizer_finish_switch_fiber(fake, nullptr, nullptr);
#endif
    t = w->th[l];
}

template <class T>
inline unsigned long long to_bits(T v) {
    static_assert(sizeof(T) <= 8, "32/64-bit shuffles only");
    unsigned long long b = 0;
    std::memcpy(&b, &v, sizeof(T));
    return b;
}

template <class T>
inline T from_bits(unsigned long long b) {
    T v;
    std::memcpy(&v, &b, sizeof(T));
    return v;
}

// Every lane publishes a word, waits for the others, then reads what it
// needs.  Two alternating slot banks make one barrier per intrinsic enough.
template <class F>
inline auto exchange(unsigned long long mine, F&& read, const std::source_location& loc) {
    Warp* w = t_warp;
    const unsigned l = lane();
    const int p = w->parity[l];
    w->slot[p][l] = mine;
    yield_lane(loc.line(), loc.file_name());
    auto r = read(w->slot[p]);
    w->parity[l] ^= 1;
    return r;
}

// Runs body(lane) for the 32 lanes of a warp on the calling host thread.
template <class Body>
inline void run_warp(Warp& w, Body& body) {
    constexpr size_t kStack = 128 << 10;  // small: ASan clears a stack's shadow on every switch
    w.stacks.assign(32 * kStack, 0);
    struct Arg {
        Warp* w;
        Body* body;
        int lane;
    };
    static thread_local Arg args[32];
    t_warp = &w;
    for (int l = 0; l < 32; ++l) {
        args[l] = {&w, &body, l};
        getcontext(&w.lane_ctx[l]);
        w.lane_ctx[l].uc_stack.ss_sp = w.stacks.data() + (size_t)l * kStack;
        w.lane_ctx[l].uc_stack.ss_size = kStack;
        w.lane_ctx[l].uc_link = &w.sched;
        auto entry = +[](unsigned hi, unsigned lo) {
            Arg* a = (Arg*)(((uintptr_t)hi << 32) | (uintptr_t)lo);
#ifdef GPM_EMU_ASAN
            __sanitizer_finish_switch_fiber(nullptr, &a->w->sched_bottom, &a->w->sched_size);
#endif
            t = a->w->th[a->lane];
            (*a->body)(a->lane);
            a->w->done[a->lane] = true;
#ifdef GPM_EMU_ASAN
            __sanitizer_start_switch_fiber(nullptr, a->w->sched_bottom, a->w->sched_size);
#endif
        };
        const uintptr_t ap = (uintptr_t)&args[l];
        makecontext(&w.lane_ctx[l], (void (*)())entry, 2, (unsigned)(ap >> 32), (unsigned)(ap & 0xffffffffu));
    }
    for (;;) {
        int finished = 0;
        for (int l = 0; l < 32; ++l) {
            if (w.done[l]) {
                ++finished;
                continue;
            }
            w.cur = l;
            t = w.th[l];
#ifdef GPM_EMU_ASAN
            void* fake = nullptr;
            __sanitizer_start_switch_fiber(&fake, w.stacks.data() + (size_t)l * kStack, kStack);
#endif
            swapcontext(&w.sched, &w.lane_ctx[l]);
#ifdef GPM_EMU_ASAN
            __sanitizer_finish_switch_fiber(fake, nullptr, nullptr);
#endif
            if (w.done[l]) ++finished;
        }
        if (finished == 32) return;
        int first = -1;
        bool mixed = false;
        for (int l = 0; l < 32; ++l) {
            if (w.done[l]) continue;
            if (first < 0) first = l;
            else if (w.site[l] != w.site[first] || w.site_file[l] != w.site_file[first]) mixed = true;
        }
        if (finished != 0 || mixed) {
            std::fprintf(stderr, "warp divergence (block %u, warp %u): %d lanes returned;", w.th[0].bid.x,
                         w.th[0].tid.x / 32, finished);
            for (int l = 0; l < 32; ++l)
                if (!w.done[l]) std::fprintf(stderr, " lane %d at %s:%u;", l, w.site_file[l] ? w.site_file[l] : "syncwarp", w.site[l]);
            std::fprintf(stderr, "\n");
            for (int l = 0; l < 32; ++l) {
                std::fprintf(stderr, "lane %2d history:", l);
                for (unsigned i = 16; i >= 1; --i)
                    if (w.nhist[l] >= i) std::fprintf(stderr, " %u", w.hist[l][(w.nhist[l] - i) & 15]);
                std::fprintf(stderr, "\n");
            }
            std::fflush(stderr);
            std::_Exit(5);
        }
    }
}

}  // namespace gpm_emu

#define threadIdx (gpm_emu::t.tid)
#define blockIdx (gpm_emu::t.bid)
#define blockDim (gpm_emu::block_dim)
#define gridDim (gpm_emu::grid_dim)

template <class A, class B>
inline typename std::common_type<A, B>::type min(A a, B b) {
    typedef typename std::common_type<A, B>::type C;
    return (C)a < (C)b ? (C)a : (C)b;
}
template <class A, class B>
inline typename std::common_type<A, B>::type max(A a, B b) {
    typedef typename std::common_type<A, B>::type C;
    return (C)a < (C)b ? (C)b : (C)a;
}

using gpm_emu_loc = std::source_location;

// the matcher never meets different __syncwarp sites, so they are checked too
inline void __syncwarp(unsigned = 0xffffffffu, gpm_emu_loc loc = gpm_emu_loc::current()) {
    gpm_emu::yield_lane(loc.line(), loc.file_name());
}

template <class T>
inline T __shfl_sync(unsigned, T v, int src, int = 32, gpm_emu_loc loc = gpm_emu_loc::current()) {
    const unsigned s = (unsigned)src & 31u;
    return gpm_emu::from_bits<T>(
        gpm_emu::exchange(gpm_emu::to_bits(v), [&](const unsigned long long* w) { return w[s]; }, loc));
}
template <class T>
inline T __shfl_xor_sync(unsigned, T v, int m, int = 32, gpm_emu_loc loc = gpm_emu_loc::current()) {
    const unsigned s = (gpm_emu::lane() ^ (unsigned)m) & 31u;
    return gpm_emu::from_bits<T>(
        gpm_emu::exchange(gpm_emu::to_bits(v), [&](const unsigned long long* w) { return w[s]; }, loc));
}
template <class T>
inline T __shfl_up_sync(unsigned, T v, unsigned delta, int = 32, gpm_emu_loc loc = gpm_emu_loc::current()) {
    const unsigned l = gpm_emu::lane();
    const unsigned s = l >= delta ? l - delta : l;
    return gpm_emu::from_bits<T>(
        gpm_emu::exchange(gpm_emu::to_bits(v), [&](const unsigned long long* w) { return w[s]; }, loc));
}
inline unsigned __ballot_sync(unsigned, int pred, gpm_emu_loc loc = gpm_emu_loc::current()) {
    return gpm_emu::exchange(
        pred ? 1ull : 0ull,
        [](const unsigned long long* w) {
            unsigned m = 0;
            for (int i = 0; i < 32; ++i) m |= (w[i] ? 1u : 0u) << i;
            return m;
        },
        loc);
}
inline int __all_sync(unsigned mask, int pred, gpm_emu_loc loc = gpm_emu_loc::current()) {
    return __ballot_sync(mask, pred, loc) == 0xffffffffu;
}
template <class T>
inline unsigned __match_any_sync(unsigned, T v, gpm_emu_loc loc = gpm_emu_loc::current()) {
    const unsigned long long mine = gpm_emu::to_bits(v);
    return gpm_emu::exchange(
        mine,
        [&](const unsigned long long* w) {
            unsigned m = 0;
            for (int i = 0; i < 32; ++i) m |= (w[i] == mine ? 1u : 0u) << i;
            return m;
        },
        loc);
}

inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }
inline int __clz(int x) { return x == 0 ? 32 : __builtin_clz((unsigned)x); }

inline void __threadfence() { __atomic_thread_fence(__ATOMIC_SEQ_CST); }
template <class T>
inline T __ldcg(const T* p) { return __atomic_load_n(p, __ATOMIC_RELAXED); }
inline void __nanosleep(unsigned) { std::this_thread::yield(); }

template <class T>
inline T atomicAdd(T* p, T v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
template <class T>
inline T atomicOr(T* p, T v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
template <class T>
inline T atomicExch(T* p, T v) { return __atomic_exchange_n(p, v, __ATOMIC_SEQ_CST); }
template <class T>
inline T atomicCAS(T* p, T cmp, T v) {
    __atomic_compare_exchange_n(p, &cmp, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST);
    return cmp;
}
