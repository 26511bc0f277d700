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

#include "match_core.cuh"

// Bytes allocated past the end of every neighbour array and scratch area:
// a bulk copy of a staged set covers the 16-byte aligned span around it.
constexpr size_t kCsrSlack = 16;

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

// k-clique counting, the clique fast path: Graph::pattern_matching_func with
// clique = true (src/graph.cpp:147-197) and VertexSet::intersection's
// min_vertex clip (src/vertex_set.cpp:75-103) for a complete pattern.  Every
// clique is counted once, as its decreasing vertex sequence v0 > v1 > ...:
// a task is a directed edge (v0, v1) with v1 < v0, S0 = N(v0) ∩ N(v1) below
// v1, and below that S_{d+1} = S_d[0, i) ∩ N(S_d[i]) — the members of S_d
// before position i are exactly those below S_d[i], so the clip is an index.
// The last level counts |S_d[0, i) ∩ N(S_d[i])| without writing it.  No
// restriction bounds or injectivity checks are needed: the order implies
// both.  One warp per task; sets of level d live in the warp's scratch slot d.
__global__ void __launch_bounds__(256) clique_kernel(GraphView g, int k, unsigned long long* __restrict__ cursor,
                                                     unsigned long long* __restrict__ out, int* __restrict__ scratch,
                                                     int cap, int chunk, const unsigned long long* __restrict__ params) {
    const unsigned long long stripes = params[0], stripe = params[1];
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int* base = scratch + (size_t)gw * (size_t)max(1, k - 3) * (size_t)cap;
    __int128 acc = 0;
    int cur_v = -1;
    unsigned cur_lo = 0, cur_hi = 0;
    int idx[kMaxN], len[kMaxN];
    for (;;) {
        unsigned long long q = 0;
        if (lane == 0) q = atomicAdd(cursor, 1ull);
        q = __shfl_sync(kFull, q, 0);
        const unsigned long long i0 = q * (unsigned long long)chunk;
        if (i0 * stripes + stripe >= g.e_cnt) break;
        for (unsigned long long i = i0; i < i0 + (unsigned long long)chunk; ++i) {
            const unsigned long long t = i * stripes + stripe;
            if (t >= g.e_cnt) break;
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
            const int v1 = g.col[e];
            if ((unsigned)v1 >= (unsigned)g.v_cnt) {
                if (lane == 0) record_check(kErrBadVertex, e, v1, cur_v, g.v_cnt, 0, 0);
                continue;
            }
            if (v1 >= cur_v) continue;
            const int* n0 = g.col + cur_lo;
            const int* n1 = g.col + g.rowptr[v1];
            const int d1 = (int)(g.rowptr[v1 + 1] - g.rowptr[v1]);
            if (k == 3) {
                acc += isect_count(n0, (int)(cur_hi - cur_lo), n1, d1, v1, nullptr, 0, lane);
                continue;
            }
            const int na = lower_bound_u(n0, (int)(cur_hi - cur_lo), v1);
            const int nb = lower_bound_u(n1, d1, v1);
            if (min(na, nb) > cap) {
                if (lane == 0) record_check(kErrSetSize, -1, na, nb, cap, 0, 0);
                continue;
            }
            len[0] = isect_store(n0, na, n1, nb, base, lane);
            idx[0] = 0;
            int d = 0;
            while (d >= 0) {
                if (idx[d] >= len[d]) {
                    --d;
                    continue;
                }
                const int* S = base + (size_t)d * cap;
                const int pos = idx[d]++;
                const int w = S[pos];
                if ((unsigned)w >= (unsigned)g.v_cnt) {
                    if (lane == 0) record_check(kErrBadVertex, w, g.v_cnt, k, d, 0, 0);
                    continue;
                }
                const int* nw = g.col + g.rowptr[w];
                const int dw = (int)(g.rowptr[w + 1] - g.rowptr[w]);
                if (d == k - 4) {  // the last vertex: count, do not store
                    acc += isect_count(S, pos, nw, dw, w, nullptr, 0, lane);
                    continue;
                }
                len[d + 1] = isect_store(S, pos, nw, lower_bound_u(nw, dw, w), base + (size_t)(d + 1) * cap, lane);
                if (len[d + 1] > 0) {
                    idx[d + 1] = 0;
                    ++d;
                }
            }
        }
    }
    if (lane == 0 && acc != 0) add128(out, acc);
}

#include "csr_rows.cuh"

// CSR checks in one streaming pass (the graph's own load-time checks): the
// offsets are nondecreasing and end at e_cnt (each vertex, one thread);
// then the edge positions in chunks of kValidateChunk per warp, each
// position's row found by csr_batch_row: ids in range, no self loops,
// lists strictly increasing, and symmetry — the sum over edges of a 64-bit
// mix of (u, v) equals the sum of the mix of (v, u) exactly when every edge
// has its reverse (as multisets; duplicates are already excluded), under
// two salts so that a false match needs two independent 64-bit sums to
// collide (about 2^-128 for any fixed input).  words[0]: flag bits
// (atomicOr on its low word), words[1..4]: the sums.  The position pass
// reads rows only through the offsets, which stay in [0, V) even when they
// are malformed (flag 1 then reports it).
constexpr unsigned kValidateChunk = 4096;
__device__ __forceinline__ unsigned long long edge_mix(unsigned long long key, unsigned long long salt) {
    unsigned long long z = key + salt;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
constexpr unsigned long long kSalt1 = 0x9E3779B97F4A7C15ull, kSalt2 = 0xD1B54A32D192ED03ull;

__global__ void validate_kernel(GraphView g, unsigned long long* __restrict__ words) {
    const int lane = threadIdx.x & 31;
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    unsigned bad = 0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < g.v_cnt; v += nthreads) {
        const unsigned a = g.rowptr[v], b = g.rowptr[v + 1];
        if (b < a || b > g.e_cnt) bad |= 1;
    }
    unsigned long long f1 = 0, b1 = 0, f2 = 0, b2 = 0;
    const unsigned long long E = g.e_cnt;
    const long long nw = nthreads >> 5;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (unsigned long long c0 = (unsigned long long)w0 * kValidateChunk; c0 < E;
         c0 += (unsigned long long)nw * kValidateChunk) {
        const unsigned long long c1 = min(E, c0 + kValidateChunk);
        int r0 = 0;
        if (lane == 0) r0 = csr_row_of(g.rowptr, g.v_cnt, c0);
        r0 = __shfl_sync(kFull, r0, 0);
        for (unsigned long long kb = c0; kb < c1; kb += 32) {
            const int row = csr_batch_row(g.rowptr, g.v_cnt, kb, c1, r0, lane);
            const unsigned long long k = kb + (unsigned long long)lane;
            const int x = k < c1 ? g.col[k] : 0;
            const int left = __shfl_up_sync(kFull, x, 1);
            if (k < c1) {
                if (x < 0 || x >= g.v_cnt) {
                    bad |= 2;
                } else {
                    if (x == row) bad |= 4;
                    if (k > (unsigned long long)g.rowptr[row]) {
                        const int prev = lane ? left : g.col[k - 1];
                        if (prev >= x) bad |= 8;
                    }
                    const unsigned long long kf = ((unsigned long long)(unsigned)row << 32) | (unsigned)x;
                    const unsigned long long kr = ((unsigned long long)(unsigned)x << 32) | (unsigned)row;
                    f1 += edge_mix(kf, kSalt1);
                    b1 += edge_mix(kr, kSalt1);
                    f2 += edge_mix(kf, kSalt2);
                    b2 += edge_mix(kr, kSalt2);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        f1 += __shfl_xor_sync(kFull, f1, o);
        b1 += __shfl_xor_sync(kFull, b1, o);
        f2 += __shfl_xor_sync(kFull, f2, o);
        b2 += __shfl_xor_sync(kFull, b2, o);
    }
    if (bad) atomicOr(reinterpret_cast<unsigned*>(words), bad);
    if (lane == 0) {
        atomicAdd(words + 1, f1);
        atomicAdd(words + 2, b1);
        atomicAdd(words + 3, f2);
        atomicAdd(words + 4, b2);
    }
}

// flag bits of a validate_kernel result (16: not symmetric)
static unsigned csr_flags(const unsigned long long* w) {
    unsigned f = (unsigned)(w[0] & 0xffffffffull);
    if (w[1] != w[2] || w[3] != w[4]) f |= 16;
    return f;
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

// The relabelled edges in new-row order, unsorted within a row: output
// position p of new row i (old vertex order[i]) takes the new id of the old
// list's element at the same offset, and src[p] = i.  Positions go in
// chunks per warp as in validate_kernel.
__global__ void relabel_fill_kernel(const unsigned* __restrict__ rowptr, const int* __restrict__ col,
                                    const int* __restrict__ order, const int* __restrict__ new_id,
                                    const unsigned* __restrict__ new_rowptr, int v_cnt, unsigned long long e_cnt,
                                    unsigned* __restrict__ out, int* __restrict__ src) {
    const int lane = threadIdx.x & 31;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    for (unsigned long long c0 = (unsigned long long)w0 * kValidateChunk; c0 < e_cnt;
         c0 += (unsigned long long)nw * kValidateChunk) {
        const unsigned long long c1 = min(e_cnt, c0 + kValidateChunk);
        int r0 = 0;
        if (lane == 0) r0 = csr_row_of(new_rowptr, v_cnt, c0);
        r0 = __shfl_sync(kFull, r0, 0);
        for (unsigned long long pb = c0; pb < c1; pb += 32) {
            const int i = csr_batch_row(new_rowptr, v_cnt, pb, c1, r0, lane);
            const unsigned long long q = pb + (unsigned long long)lane;
            if (q < c1) {
                const int o = order[i];
                const unsigned long long k = (unsigned long long)rowptr[o] + (q - new_rowptr[i]);
                out[q] = (unsigned)new_id[col[k]];
                src[q] = i;
            }
        }
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
    cudaMemPool_t pool = nullptr;  // graph arrays and construction temporaries (null: cudaMalloc)
    // the dense counter arrays of the scratch known to be zero (every pair
    // sum zeroes what it counted; a failed launch or another use of the
    // scratch clears this, and the next launch zeroes the arrays again)
    const void* dense_clean = nullptr;
    size_t dense_clean_bytes = 0;
    const void* tables_clean = nullptr;  // likewise the pair-sum tables and their stored tags
    size_t tables_clean_bytes = 0;
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
        // A stream-ordered pool that keeps freed memory (up to a quarter of
        // the device) for the next call, so that a graph uploaded per call
        // does not map and unmap its buffers every time.  Without it (an
        // error here, or option pool=0) buffers come from cudaMalloc.
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = t_device;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess && cudaMemPoolCreate(&nc->pool, &props) == cudaSuccess) {
            unsigned long long keep = (unsigned long long)(total_b / 4);
            if (cudaMemPoolSetAttribute(nc->pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
                cudaMemPoolDestroy(nc->pool);
                nc->pool = nullptr;
            }
        } else {
            nc->pool = nullptr;
        }
        cudaGetLastError();
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
    c->dense_clean = nullptr;
    c->dense_clean_bytes = 0;
    c->tables_clean = nullptr;
    c->tables_clean_bytes = 0;
    if (c->scratch) cudaFree(c->scratch);
    c->scratch = nullptr;
    c->scratch_bytes = 0;
    GPM_CK(cudaMalloc(&c->scratch, bytes));
    c->scratch_bytes = bytes;
    return GPM_OK;
}

// RAII device buffer for one call
static bool use_pool(const DeviceCtx* c) { return c->pool != nullptr && options().pool != 0; }

static cudaError_t buf_alloc(DeviceCtx* c, void** p, size_t bytes, bool pooled) {
    return pooled ? cudaMallocFromPoolAsync(p, bytes, c->pool, c->stream) : cudaMalloc(p, bytes);
}

// frees a buffer of buf_alloc (stream-ordered on the context's stream when pooled)
static void buf_free(void* p, bool pooled, cudaStream_t st) {
    if (!p) return;
    if (pooled) cudaFreeAsync(p, st);
    else cudaFree(p);
}

struct DevBuf {
    void* p = nullptr;
    bool pooled = false;
    cudaStream_t st = nullptr;
    cudaError_t alloc(DeviceCtx* c, size_t bytes) { return alloc(c, bytes, use_pool(c)); }
    cudaError_t alloc(DeviceCtx* c, size_t bytes, bool from_pool) {
        pooled = from_pool;
        st = c->stream;
        return buf_alloc(c, &p, bytes, pooled);
    }
    ~DevBuf() { buf_free(p, pooled, st); }
};

// The graph's device arrays.  With pooled arrays the device is synchronised
// first, as cudaFree would: no kernel on any stream reads them any more.
static void graph_free_arrays(gpm_graph* g) {
    void* ps[4] = {g->orig_rowptr != g->rowptr ? (void*)g->orig_rowptr : nullptr,
                   g->orig_col != g->col ? (void*)g->orig_col : nullptr, g->rowptr, g->col};
    if (g->pooled) cudaDeviceSynchronize();
    for (void* q : ps) buf_free(q, g->pooled, (cudaStream_t)g->stream);
    g->orig_rowptr = g->rowptr = nullptr;
    g->orig_col = g->col = nullptr;
}

static cudaError_t graph_alloc(DeviceCtx* c, gpm_graph* g, void** p, size_t bytes) {
    return buf_alloc(c, p, bytes, g->pooled);
}

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
    GPM_CK(keys.alloc(c, sizeof(unsigned) * (size_t)std::max(V, 1)));
    GPM_CK(keys2.alloc(c, sizeof(unsigned) * (size_t)std::max(V, 1)));
    GPM_CK(ids.alloc(c, sizeof(int) * (size_t)std::max(V, 1)));
    GPM_CK(order.alloc(c, sizeof(int) * (size_t)std::max(V, 1)));
    const int threads = 256, blocks = c->num_sms * 8;
    degree_keys_kernel<<<blocks, threads, 0, st>>>(g->rowptr, V, (unsigned*)keys.p, (int*)ids.p);
    GPM_CK(cudaGetLastError());
    size_t tb = 0;
    GPM_CK(cub::DeviceRadixSort::SortPairs(nullptr, tb, (unsigned*)keys.p, (unsigned*)keys2.p, (int*)ids.p,
                                           (int*)order.p, V, 0, 32, st));
    GPM_CK(tmp.alloc(c, std::max<size_t>(tb, 1)));
    GPM_CK(cub::DeviceRadixSort::SortPairs(tmp.p, tb, (unsigned*)keys.p, (unsigned*)keys2.p, (int*)ids.p,
                                           (int*)order.p, V, 0, 32, st));
    unsigned top[2] = {~0u, ~0u};
    GPM_CK(cudaMemcpyAsync(top, keys2.p, sizeof(unsigned) * std::min(V, 2), cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    g->max_degree = V >= 1 ? (int)~top[0] : 0;
    g->max_isect = V >= 2 ? (int)~top[1] : g->max_degree;
    if (!relabel || V == 0 || E == 0) return GPM_OK;

    // The relabelled lists come out sorted from one stable radix sort of the
    // edges (new source i, new destination j) by j: the fill writes them in
    // increasing i, and the graph is symmetric, so row j of the result lists
    // its neighbours i in increasing order.
    DevBuf new_id, new_deg, new_rowptr, keys_a, keys_b, vals_a, vals_b, tmp2;
    GPM_CK(new_id.alloc(c, sizeof(int) * (size_t)V));
    GPM_CK(new_deg.alloc(c, sizeof(unsigned) * ((size_t)V + 1)));
    GPM_CK(new_rowptr.alloc(c, sizeof(unsigned) * ((size_t)V + 1), g->pooled));
    GPM_CK(keys_a.alloc(c, sizeof(unsigned) * (size_t)E));
    GPM_CK(keys_b.alloc(c, sizeof(unsigned) * (size_t)E));
    GPM_CK(vals_a.alloc(c, sizeof(int) * (size_t)E + kCsrSlack, g->pooled));
    GPM_CK(vals_b.alloc(c, sizeof(int) * (size_t)E + kCsrSlack, g->pooled));
    relabel_maps_kernel<<<blocks, threads, 0, st>>>(g->rowptr, (const int*)order.p, V, (int*)new_id.p,
                                                    (unsigned*)new_deg.p);
    GPM_CK(cudaGetLastError());
    size_t sb = 0;
    GPM_CK(cub::DeviceScan::ExclusiveSum(nullptr, sb, (unsigned*)new_deg.p, (unsigned*)new_rowptr.p, V + 1, st));
    GPM_CK(tmp2.alloc(c, std::max<size_t>(sb, 1)));
    GPM_CK(cub::DeviceScan::ExclusiveSum(tmp2.p, sb, (unsigned*)new_deg.p, (unsigned*)new_rowptr.p, V + 1, st));
    relabel_fill_kernel<<<blocks, threads, 0, st>>>(g->rowptr, g->col, (const int*)order.p, (const int*)new_id.p,
                                                    (const unsigned*)new_rowptr.p, V, (unsigned long long)E,
                                                    (unsigned*)keys_a.p, (int*)vals_a.p);
    GPM_CK(cudaGetLastError());
    int end_bit = 1;
    while (end_bit < 32 && (1ull << end_bit) < (unsigned long long)V) ++end_bit;
    cub::DoubleBuffer<unsigned> dkeys((unsigned*)keys_a.p, (unsigned*)keys_b.p);
    cub::DoubleBuffer<int> dvals((int*)vals_a.p, (int*)vals_b.p);
    size_t ssb = 0;
    GPM_CK(cub::DeviceRadixSort::SortPairs(nullptr, ssb, dkeys, dvals, (unsigned long long)E, 0, end_bit, st));
    DevBuf tmp3;
    GPM_CK(tmp3.alloc(c, std::max<size_t>(ssb, 1)));
    GPM_CK(cub::DeviceRadixSort::SortPairs(tmp3.p, ssb, dkeys, dvals, (unsigned long long)E, 0, end_bit, st));
    DevBuf& new_col = dvals.Current() == (int*)vals_a.p ? vals_a : vals_b;
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
    DevBuf buf;
    unsigned long long w[5] = {0, 0, 0, 0, 0};
    *rc = GPM_OK;
    if (buf.alloc(c, sizeof w) != cudaSuccess) {
        set_error("validate: out of device memory");
        *rc = GPM_ERR_OOM;
        return 0;
    }
    unsigned long long* d_words = (unsigned long long*)buf.p;
    cudaMemsetAsync(d_words, 0, sizeof w, c->stream);
    validate_kernel<<<c->num_sms * 8, 256, 0, c->stream>>>(v, d_words);
    cudaMemcpyAsync(w, d_words, sizeof w, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        set_error("validate: %s", cudaGetErrorString(e));
        *rc = GPM_ERR_CUDA;
        return 0;
    }
    return csr_flags(w);
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

// Pair-sum tables: 2^pair_log2 64-bit words per warp (2^17 unless forced or
// a quarter of the free memory left after the set slots is less).
constexpr int kPairLog2Min = 13, kPairLog2Default = 17;

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
    int pair_log2 = kPairLog2Min;
    int split_min = 0;
    int bm_words = 0;  // words per leaf bitmap (0: no bitmaps)
    int bm_min = 0;
    int min_blocks = 1;  // kernel variant: 1, 3 or 4 resident blocks per SM
    int dense_slots = 0;  // pool of per-vertex counter arrays for big pair sums
    int dense_words = 0;
    bool count_bytes = false;
};


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
    // the stage holds fixed sets of the batched leaf only: without it, no
    // shared memory goes to staging (more blocks fit an SM)
    ls.stage_cap = o.leaf_batch ? (int)o.stage_max : 0;
    ls.smem = sizeof(WarpState) * ls.wpb + sizeof(int) * 2 * (size_t)stage_stride(ls.stage_cap) * ls.wpb;
    ls.count_bytes = o.count_bytes != 0;
    ls.min_blocks = ((o.min_blocks >= 3 && o.min_blocks <= 5) && !ls.count_bytes) ? (int)o.min_blocks : 1;
    if (ls.min_blocks > 1 && ls.wpb > (ls.min_blocks == 5 ? 4 : 8)) {
        set_error("min_blocks=%d needs warps_per_block <= %d (got %d)", ls.min_blocks, ls.min_blocks == 5 ? 4 : 8,
                  ls.wpb);
        return GPM_ERR_INVALID_ARG;
    }
    const void* kfn = ls.count_bytes       ? (const void*)match_kernel<true, 1>
                      : ls.min_blocks == 5 ? (const void*)match_kernel<false, 5>
                      : ls.min_blocks == 4 ? (const void*)match_kernel<false, 4>
                      : ls.min_blocks == 3 ? (const void*)match_kernel<false, 3>
                                           : (const void*)match_kernel<false, 1>;
    GPM_CK(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ls.smem));
    // a persistent grid: no more blocks than can be resident at once
    int occ = 0;
    GPM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kfn, ls.wpb * 32, ls.smem));
    if (occ < 1) {
        set_error("launch shape does not fit an SM: %d warps per block, %zu bytes of shared memory", ls.wpb, ls.smem);
        return GPM_ERR_INVALID_ARG;
    }
    // the 3-block variant launches three blocks per SM when they fit
    ls.blocks = (long long)c->num_sms * std::min<long long>(std::max<long long>(o.blocks_per_sm, ls.min_blocks), occ);
    // set slots, then the pair sums' two block-sum arrays at the end
    ls.per_warp = (long long)nslots * cap + 2 * pair_bs_stride(cap);
    // shrink the grid when the per-warp scratch would not fit in free memory
    size_t free_b = 0, total_b = 0;
    GPM_CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = (size_t)((free_b + scratch_budget_extra) * 0.6);
    while (ls.blocks > 1 && (size_t)ls.blocks * ls.wpb * ls.per_warp * sizeof(int) > budget)
        ls.blocks = (ls.blocks + 1) / 2;
    const int alpha4[3] = {(int)o.merge_alpha4[0], (int)o.merge_alpha4[1], (int)o.merge_alpha4[2]};
    GPM_CK(cudaMemcpyToSymbolAsync(c_merge_alpha4, alpha4, sizeof alpha4, 0, cudaMemcpyHostToDevice, c->stream));
    const int mvec = (int)o.merge_vec;
    GPM_CK(cudaMemcpyToSymbolAsync(c_merge_vec, &mvec, sizeof mvec, 0, cudaMemcpyHostToDevice, c->stream));
    const long long pair_max = (long long)o.pair_max_ops;
    GPM_CK(cudaMemcpyToSymbolAsync(c_pair_max_ops, &pair_max, sizeof pair_max, 0, cudaMemcpyHostToDevice, c->stream));
    // A grab takes `chunk` tasks of the stripe, but never leaves warps
    // without a task: when a stripe holds fewer than chunk tasks per warp
    // (thin benchmark stripes), grabs shrink down to one task.
    {
        const unsigned long long warps = (unsigned long long)ls.blocks * ls.wpb;
        const unsigned long long stripes = (unsigned long long)std::max<int64_t>(1, o.stripes);
        unsigned long long fewest = ~0ull;
        for (const PairDesc& d : ls.descs) fewest = std::min(fewest, (d.ntasks + stripes - 1) / stripes);
        ls.chunk = (int)std::max<unsigned long long>(1, std::min<unsigned long long>(o.chunk, fewest / warps));
    }
    // bit 1: stage fixed sets with bulk copies (their sources carry the slack)
    ls.leaf_on = (int)o.leaf_batch | (o.stage_tma ? 2 : 0);
    ls.pair_on = 0;
    if (o.pair_leaf) {
        bool any = false;
        for (int i = 0; i < n; ++i) any |= plans[i]->host.pair_ok && graphs[i]->v_cnt <= (1 << 24);
        ls.pair_on = any ? 1 : 0;
    }
    if (ls.pair_on) {
        const size_t warps = (size_t)ls.blocks * ls.wpb;
        const size_t sets = warps * (size_t)ls.per_warp * sizeof(int);
        const size_t room = (free_b + scratch_budget_extra) > sets ? (free_b + scratch_budget_extra - sets) / 4 : 0;
        if (o.pair_log2) {
            ls.pair_log2 = (int)o.pair_log2;
        } else {
            // a fixed size (1 MB per warp), smaller only when memory is short:
            // pair sums too big for it run on the shared dense arrays
            ls.pair_log2 = kPairLog2Default;
            while (ls.pair_log2 > kPairLog2Min && warps * ((size_t)8 << ls.pair_log2) > room) --ls.pair_log2;
        }
        // dense counter arrays for the pair sums too big for a table: up to
        // 64, within an eighth of the free memory
        int vmax = 0;
        for (int i = 0; i < n; ++i) vmax = std::max(vmax, graphs[i]->v_cnt);
        ls.dense_words = vmax;
        ls.dense_slots = (int)std::min<int64_t>(o.dense_slots, (int64_t)(room / 2 / ((size_t)vmax * 4 + 1)));
        if (ls.dense_slots < 1) ls.dense_slots = 0;
    }
    ls.split_min = (int)o.split;
    // two bitmaps over vertex ids per warp for the batched leaves
    ls.bm_words = 0;
    ls.bm_min = (int)o.bitmap_min;
    if ((ls.leaf_on & 1) && ls.bm_min > 0) {
        int vmax = 0;
        bool any = false;
        for (int i = 0; i < n; ++i) {
            vmax = std::max(vmax, graphs[i]->v_cnt);
            any |= plans[i]->host.leaf_kind != kLeafGeneric;
        }
        const size_t words = ((size_t)vmax + 31) / 32;
        const size_t warps = (size_t)ls.blocks * ls.wpb;
        if (any && warps * 2 * words * sizeof(unsigned) <= (free_b + scratch_budget_extra) / 8) ls.bm_words = (int)words;
    }
    return GPM_OK;
}

// small device words of a launch: cursors[n], out[2n], stats[2], params[2]
static size_t small_words(int n) { return (size_t)n * 3 + 4; }

// Scratch of a launch: per-warp set slots, per-warp pair tables, then the
// donation records (zeroed before every launch).
struct ScratchLayout {
    size_t tables = 0, donation = 0, bitmaps = 0, dense = 0, total = 0;
};

// lock words padded to 64, then dense_slots arrays of dense_words counters
static size_t dense_bytes(const LaunchSetup& ls) {
    if (!ls.dense_slots) return 0;
    return (((size_t)ls.dense_slots + 63) & ~(size_t)63) * sizeof(unsigned) +
           (size_t)ls.dense_slots * ls.dense_words * sizeof(unsigned);
}

static size_t bitmap_bytes(const LaunchSetup& ls) {
    return (size_t)ls.blocks * ls.wpb * 2 * (size_t)ls.bm_words * sizeof(unsigned);
}

// the warps' pair-sum tables, then one stored tag per warp (kept across
// launches: zeroed only when new or after a failed launch)
static size_t pair_region_bytes(const LaunchSetup& ls) {
    const size_t warps = (size_t)ls.blocks * ls.wpb;
    return warps * ((size_t)1 << ls.pair_log2) * sizeof(unsigned long long) + ((warps * sizeof(unsigned) + 255) & ~(size_t)255);
}

static ScratchLayout scratch_layout(const LaunchSetup& ls) {
    const size_t warps = (size_t)ls.blocks * ls.wpb;
    ScratchLayout s;
    size_t b = warps * (size_t)ls.per_warp * sizeof(int);
    b = (b + 255) & ~(size_t)255;
    s.tables = b;
    if (ls.pair_on) b += pair_region_bytes(ls);
    s.donation = b;
    if (ls.split_min > 0) b += sizeof(DonationArea);
    b = (b + 255) & ~(size_t)255;
    s.bitmaps = b;
    b += bitmap_bytes(ls);
    b = (b + 255) & ~(size_t)255;
    s.dense = b;
    b += dense_bytes(ls);
    s.total = b + kCsrSlack;  // bulk copies of sets may round their end up by 12 bytes
    return s;
}

static size_t scratch_bytes(const LaunchSetup& ls) { return scratch_layout(ls).total; }

// zero_dense / zero_tables: zero the dense counter arrays / the pair-sum
// tables and tags first (they are new, or a failed launch may have left
// counts in them)
static cudaError_t enqueue_match(const LaunchSetup& ls, int n, const PairDesc* d_pairs,
                                 unsigned long long* d_small, int* scratch, bool zero_dense, bool zero_tables,
                                 cudaStream_t st) {
    unsigned long long* cursors = d_small;
    unsigned long long* out = cursors + n;
    unsigned long long* stats = out + 2 * n;
    const unsigned long long* params = stats + 2;
    const ScratchLayout lay = scratch_layout(ls);
    unsigned long long* tables = ls.pair_on ? (unsigned long long*)((char*)scratch + lay.tables) : nullptr;
    if (tables && zero_tables) {
        const cudaError_t e = cudaMemsetAsync(tables, 0, pair_region_bytes(ls), st);
        if (e != cudaSuccess) return e;
    }
    DonationArea* don = ls.split_min > 0 ? (DonationArea*)((char*)scratch + lay.donation) : nullptr;
    if (don) {
        const cudaError_t e = cudaMemsetAsync(don, 0, sizeof(DonationArea), st);
        if (e != cudaSuccess) return e;
    }
    unsigned* bitmaps = ls.bm_words ? (unsigned*)((char*)scratch + lay.bitmaps) : nullptr;
    if (bitmaps) {
        const cudaError_t e = cudaMemsetAsync(bitmaps, 0, bitmap_bytes(ls), st);
        if (e != cudaSuccess) return e;
    }
    unsigned* dense = ls.dense_slots ? (unsigned*)((char*)scratch + lay.dense) : nullptr;
    if (dense && zero_dense) {
        const cudaError_t e = cudaMemsetAsync(dense, 0, dense_bytes(ls), st);
        if (e != cudaSuccess) return e;
    }
#define GPM_MATCH_ARGS                                                                                        \
    d_pairs, n, cursors, out, scratch, ls.per_warp, ls.chunk, params, ls.leaf_on, ls.stage_cap, ls.pair_on, tables, \
        ls.pair_log2, don, ls.split_min, bitmaps, ls.bm_words, ls.bm_min, dense, ls.dense_slots, ls.dense_words, stats
    if (ls.count_bytes)
        match_kernel<true, 1><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(GPM_MATCH_ARGS);
    else if (ls.min_blocks == 5)
        match_kernel<false, 5><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(GPM_MATCH_ARGS);
    else if (ls.min_blocks == 4)
        match_kernel<false, 4><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(GPM_MATCH_ARGS);
    else if (ls.min_blocks == 3)
        match_kernel<false, 3><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(GPM_MATCH_ARGS);
    else
        match_kernel<false, 1><<<(unsigned)ls.blocks, ls.wpb * 32, ls.smem, st>>>(GPM_MATCH_ARGS);
#undef GPM_MATCH_ARGS
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
    GPM_CK(d_pairs.alloc(c, sizeof(PairDesc) * n));
    const size_t words = small_words(n);
    GPM_CK(d_small.alloc(c, words * sizeof(unsigned long long)));
    cudaStream_t st = c->stream;
    std::vector<unsigned long long> init(words, 0);
    init[3 * n + 2] = (unsigned long long)options().stripes;
    init[3 * n + 3] = (unsigned long long)options().stripe;
    GPM_CK(cudaMemcpyAsync(d_pairs.p, ls.descs.data(), sizeof(PairDesc) * n, cudaMemcpyHostToDevice, st));
    GPM_CK(cudaMemcpyAsync(d_small.p, init.data(), words * sizeof(unsigned long long), cudaMemcpyHostToDevice, st));
    const void* dense_ptr = ls.dense_slots ? (const char*)c->scratch + scratch_layout(ls).dense : nullptr;
    const size_t dbytes = dense_bytes(ls);
    const bool zero = dense_ptr && !(c->dense_clean == dense_ptr && c->dense_clean_bytes == dbytes);
    const void* tab_ptr = ls.pair_on ? (const char*)c->scratch + scratch_layout(ls).tables : nullptr;
    const size_t tbytes = ls.pair_on ? pair_region_bytes(ls) : 0;
    const bool zero_tab = tab_ptr && !(c->tables_clean == tab_ptr && c->tables_clean_bytes == tbytes);
    c->dense_clean = nullptr;  // until this launch has finished cleanly
    c->dense_clean_bytes = 0;
    c->tables_clean = nullptr;
    c->tables_clean_bytes = 0;
    GPM_CK(cudaEventRecord(c->ev0, st));
    GPM_CK(enqueue_match(ls, n, (const PairDesc*)d_pairs.p, (unsigned long long*)d_small.p, (int*)c->scratch, zero,
                         zero_tab, st));
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
    rc = take_check("pattern matching");
    if (rc == GPM_OK) {
        c->dense_clean = dense_ptr;
        c->dense_clean_bytes = dense_ptr ? dbytes : 0;
        c->tables_clean = tab_ptr;
        c->tables_clean_bytes = tbytes;
    }
    return rc;
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

// Validates a freshly built device CSR and relabels it by degree.
static int finish_graph(DeviceCtx* c, gpm_graph* g, bool relabel, const char* who) {
    cudaStream_t st = c->stream;
    DevBuf d_words;
    unsigned long long w[5] = {0, 0, 0, 0, 0};
    GPM_CK(d_words.alloc(c, sizeof w));
    GPM_CK(cudaMemsetAsync(d_words.p, 0, sizeof w, st));
    validate_kernel<<<c->num_sms * 8, 256, 0, st>>>(view_of(g), (unsigned long long*)d_words.p);
    GPM_CK(cudaMemcpyAsync(w, d_words.p, sizeof w, cudaMemcpyDeviceToHost, st));
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        set_error("%s: validation failed: %s", who, cudaGetErrorString(e));
        return GPM_ERR_CUDA;
    }
    const unsigned flags = csr_flags(w);
    if (flags) {
        set_error("%s: malformed CSR (%s%s%s%s%s)", who, flags & 1 ? "offsets " : "",
                  flags & 2 ? "ids-out-of-range " : "", flags & 4 ? "self-loops " : "",
                  flags & 8 ? "unsorted-or-duplicate " : "", flags & 16 ? "asymmetric" : "");
        return GPM_ERR_INVALID_ARG;
    }
    return relabel_graph(c, g, relabel);
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
    g->pooled = use_pool(c);
    g->stream = c->stream;
    auto fail = [&](int rc) {
        graph_free_arrays(g);
        delete g;
        return rc;
    };
    cudaStream_t st = c->stream;
    if (graph_alloc(c, g, (void**)&g->rowptr, sizeof(uint32_t) * ((size_t)v_cnt + 1)) != cudaSuccess ||
        graph_alloc(c, g, (void**)&g->col, sizeof(int32_t) * std::max<size_t>(E, 1) + kCsrSlack) != cudaSuccess) {
        set_error("gpm_graph_create: out of device memory for %llu edges", (unsigned long long)E);
        return fail(GPM_ERR_OOM);
    }
    if (cudaMemcpyAsync(g->rowptr, rowptr, sizeof(uint32_t) * ((size_t)v_cnt + 1), cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        (E && cudaMemcpyAsync(g->col, col, sizeof(int32_t) * E, cudaMemcpyHostToDevice, st) != cudaSuccess)) {
        set_error("gpm_graph_create: upload failed: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(GPM_ERR_CUDA);
    }
    const int rc = finish_graph(c, g, relabel != 0, "gpm_graph_create");
    if (rc) return fail(rc);
    *out = g;
    return GPM_OK;
}

// Edge list -> CSR on the GPU (the steps of src/dataloader.cpp:129-160:
// symmetrise, drop self loops, sort, deduplicate, offsets).  Keys are
// (u << 32 | v) for both directions; a self loop or an id out of range
// becomes the sentinel ~0, which sorts last.
__global__ void edge_keys_kernel(const int* __restrict__ src, const int* __restrict__ dst, long long m, int v_cnt,
                                 unsigned long long* __restrict__ keys, unsigned* __restrict__ bad) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += (long long)gridDim.x * blockDim.x) {
        const int u = src[i], v = dst[i];
        unsigned long long k0 = ~0ull, k1 = ~0ull;
        if ((unsigned)u >= (unsigned)v_cnt || (unsigned)v >= (unsigned)v_cnt) {
            atomicOr(bad, 1u);
        } else if (u != v) {
            k0 = ((unsigned long long)(unsigned)u << 32) | (unsigned)v;
            k1 = ((unsigned long long)(unsigned)v << 32) | (unsigned)u;
        }
        keys[2 * i] = k0;
        keys[2 * i + 1] = k1;
    }
}

// rowptr[v] = first key with source >= v; col = low halves
__global__ void keys_to_csr_kernel(const unsigned long long* __restrict__ keys, unsigned long long e, int v_cnt,
                                   unsigned* __restrict__ rowptr, int* __restrict__ col) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v <= v_cnt; v += stride) {
        const unsigned long long key = (unsigned long long)v << 32;
        unsigned long long lo = 0, hi = e;
        while (lo < hi) {
            const unsigned long long mid = (lo + hi) >> 1;
            if (keys[mid] < key) lo = mid + 1;
            else hi = mid;
        }
        rowptr[v] = (unsigned)lo;
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)e; i += stride)
        col[i] = (int)(unsigned)(keys[i] & 0xffffffffull);
}

GPM_API int gpm_graph_from_edges(int32_t v_cnt, int64_t m, const int32_t* src, const int32_t* dst, int32_t relabel,
                                 gpm_graph** out) {
    clear_error();
    if (!out || v_cnt < 1 || m < 0 || (m > 0 && (!src || !dst))) {
        set_error("gpm_graph_from_edges: need v_cnt >= 1, m >= 0, src, dst and out");
        return GPM_ERR_INVALID_ARG;
    }
    if ((unsigned long long)m * 2 >= (1ull << 32)) {
        set_error("gpm_graph_from_edges: %lld edges exceed 32-bit offsets", (long long)m);
        return GPM_ERR_INVALID_ARG;
    }
    *out = nullptr;
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    cudaStream_t st = c->stream;
    const size_t n2 = (size_t)std::max<int64_t>(1, 2 * m);
    DevBuf d_src, d_dst, keys, keys2, uniq, nsel, bad, tmp;
    GPM_CK(d_src.alloc(c, sizeof(int) * std::max<int64_t>(m, 1)));
    GPM_CK(d_dst.alloc(c, sizeof(int) * std::max<int64_t>(m, 1)));
    GPM_CK(keys.alloc(c, sizeof(unsigned long long) * n2));
    GPM_CK(keys2.alloc(c, sizeof(unsigned long long) * n2));
    GPM_CK(uniq.alloc(c, sizeof(unsigned long long) * n2));
    GPM_CK(nsel.alloc(c, sizeof(unsigned long long)));
    GPM_CK(bad.alloc(c, sizeof(unsigned)));
    GPM_CK(cudaMemsetAsync(bad.p, 0, sizeof(unsigned), st));
    if (m > 0) {
        GPM_CK(cudaMemcpyAsync(d_src.p, src, sizeof(int) * m, cudaMemcpyHostToDevice, st));
        GPM_CK(cudaMemcpyAsync(d_dst.p, dst, sizeof(int) * m, cudaMemcpyHostToDevice, st));
        edge_keys_kernel<<<c->num_sms * 8, 256, 0, st>>>((const int*)d_src.p, (const int*)d_dst.p, m, v_cnt,
                                                         (unsigned long long*)keys.p, (unsigned*)bad.p);
        GPM_CK(cudaGetLastError());
    }
    const int n2i = (int)std::min<size_t>(n2, (size_t)INT_MAX);
    size_t tb_sort = 0, tb_uniq = 0;
    GPM_CK(cub::DeviceRadixSort::SortKeys(nullptr, tb_sort, (unsigned long long*)keys.p, (unsigned long long*)keys2.p,
                                          n2i, 0, 64, st));
    GPM_CK(cub::DeviceSelect::Unique(nullptr, tb_uniq, (unsigned long long*)keys2.p, (unsigned long long*)uniq.p,
                                     (unsigned long long*)nsel.p, n2i, st));
    GPM_CK(tmp.alloc(c, std::max<size_t>(std::max(tb_sort, tb_uniq), 1)));
    unsigned long long h_n = 0, h_last = ~0ull;
    unsigned h_bad = 0;
    if (m > 0) {
        GPM_CK(cub::DeviceRadixSort::SortKeys(tmp.p, tb_sort, (unsigned long long*)keys.p,
                                              (unsigned long long*)keys2.p, n2i, 0, 64, st));
        GPM_CK(cub::DeviceSelect::Unique(tmp.p, tb_uniq, (unsigned long long*)keys2.p, (unsigned long long*)uniq.p,
                                         (unsigned long long*)nsel.p, n2i, st));
        GPM_CK(cudaMemcpyAsync(&h_n, nsel.p, sizeof h_n, cudaMemcpyDeviceToHost, st));
    }
    GPM_CK(cudaMemcpyAsync(&h_bad, bad.p, sizeof h_bad, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    if (h_bad) {
        set_error("gpm_graph_from_edges: an edge names a vertex outside [0, %d)", v_cnt);
        return GPM_ERR_INVALID_ARG;
    }
    if (h_n > 0) {
        GPM_CK(cudaMemcpy(&h_last, (unsigned long long*)uniq.p + (h_n - 1), sizeof h_last, cudaMemcpyDeviceToHost));
        if (h_last == ~0ull) --h_n;  // the self-loop sentinel
    }
    gpm_graph* g = new gpm_graph();
    g->v_cnt = v_cnt;
    g->e_cnt = h_n;
    g->device = c->device;
    g->pooled = use_pool(c);
    g->stream = c->stream;
    if (graph_alloc(c, g, (void**)&g->rowptr, sizeof(uint32_t) * ((size_t)v_cnt + 1)) != cudaSuccess ||
        graph_alloc(c, g, (void**)&g->col, sizeof(int32_t) * std::max<size_t>(h_n, 1) + kCsrSlack) != cudaSuccess) {
        graph_free_arrays(g);
        delete g;
        set_error("gpm_graph_from_edges: out of device memory for %llu edges", h_n);
        return GPM_ERR_OOM;
    }
    keys_to_csr_kernel<<<c->num_sms * 8, 256, 0, st>>>((const unsigned long long*)uniq.p, h_n, v_cnt, g->rowptr,
                                                       g->col);
    const int rc = finish_graph(c, g, relabel != 0, "gpm_graph_from_edges");
    if (rc) {
        graph_free_arrays(g);
        delete g;
        return rc;
    }
    *out = g;
    return GPM_OK;
}

GPM_API int gpm_graph_download(const gpm_graph* g, uint32_t* rowptr, int32_t* col) {
    clear_error();
    if (!g || !rowptr || (g->e_cnt && !col)) {
        set_error("gpm_graph_download: null argument");
        return GPM_ERR_INVALID_ARG;
    }
    const uint32_t* rp = g->orig_rowptr ? g->orig_rowptr : g->rowptr;
    const int32_t* cl = g->orig_col ? g->orig_col : g->col;
    GPM_CK(cudaMemcpy(rowptr, rp, sizeof(uint32_t) * ((size_t)g->v_cnt + 1), cudaMemcpyDeviceToHost));
    if (g->e_cnt) GPM_CK(cudaMemcpy(col, cl, sizeof(int32_t) * g->e_cnt, cudaMemcpyDeviceToHost));
    return GPM_OK;
}

GPM_API int gpm_graph_device_csr(const gpm_graph* g, int32_t caller_ids, const uint32_t** rowptr,
                                 const int32_t** col) {
    clear_error();
    if (!g || !rowptr || !col) {
        set_error("gpm_graph_device_csr: null argument");
        return GPM_ERR_INVALID_ARG;
    }
    const GraphView v = view_of(g, caller_ids != 0);
    *rowptr = v.rowptr;
    *col = v.col;
    return GPM_OK;
}

GPM_API int gpm_graph_destroy(gpm_graph* g) {
    clear_error();
    if (!g) return GPM_OK;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(g->device);
    graph_free_arrays(g);
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
    GPM_CK(buf.alloc(c, 2 * sizeof(unsigned long long)));
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

GPM_API int gpm_clique_count(gpm_graph* g, int32_t k, gpm_u128* out) {
    clear_error();
    if (!g || !out || k < 3 || k > GPM_MAX_PATTERN) {
        set_error("gpm_clique_count: need a graph, out and 3 <= k <= %d", GPM_MAX_PATTERN);
        return GPM_ERR_INVALID_ARG;
    }
    int err = 0;
    DeviceCtx* c = get_ctx(&err);
    if (!c) return err;
    std::lock_guard<std::mutex> lk(c->mu);
    const Options& o = options();
    const int threads = 256, warps_per_block = threads / 32;
    const long long blocks = (long long)c->num_sms * 8;
    const long long warps = blocks * warps_per_block;
    const size_t per_warp = (size_t)std::max(1, k - 3) * (size_t)std::max(1, g->max_degree);
    int rc = ensure_scratch(c, warps * per_warp * sizeof(int));
    if (rc) return rc;
    c->dense_clean = nullptr;  // the clique kernel writes over the matcher's scratch
    c->dense_clean_bytes = 0;
    c->tables_clean = nullptr;
    c->tables_clean_bytes = 0;
    DevBuf buf;
    // cursor, 128-bit count, stripes, stripe
    GPM_CK(buf.alloc(c, 5 * sizeof(unsigned long long)));
    cudaStream_t st = c->stream;
    const unsigned long long init[5] = {0, 0, 0, (unsigned long long)std::max<int64_t>(1, o.stripes),
                                        (unsigned long long)o.stripe};
    GPM_CK(cudaMemcpyAsync(buf.p, init, sizeof init, cudaMemcpyHostToDevice, st));
    unsigned long long* d = (unsigned long long*)buf.p;
    const unsigned long long per_stripe = (g->e_cnt + init[3] - 1) / init[3];
    const int chunk = (int)std::max<unsigned long long>(1, std::min<unsigned long long>(o.chunk, per_stripe / warps));
    GPM_CK(cudaEventRecord(c->ev0, st));
    clique_kernel<<<(unsigned)blocks, threads, 0, st>>>(view_of(g), k, d, d + 1, (int*)c->scratch,
                                                        (int)std::max<size_t>(1, g->max_degree), chunk, d + 3);
    GPM_CK(cudaGetLastError());
    GPM_CK(cudaEventRecord(c->ev1, st));
    unsigned long long h[2] = {0, 0};
    GPM_CK(cudaMemcpyAsync(h, d + 1, sizeof h, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    t_ms = ms;
    t_launches = 1;
    t_bytes = 0;
    rc = take_check("gpm_clique_count");
    if (rc) return rc;
    out->lo = h[0];
    out->hi = h[1];
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
    bool dense_dirty = true;  // zero the dense counter arrays and pair-sum tables before the next replay
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
    const cudaError_t qe =
        enqueue_match(e->ls, n, (const PairDesc*)e->d_pairs, e->d_small, e->scratch, false, false, st);
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
    if (e->dense_dirty) {
        // the replayed launch leaves the counters zero and the tables' tags
        // current; zeroed here when new or after a failure
        if (e->ls.dense_slots)
            GPM_CK(cudaMemsetAsync((char*)e->scratch + scratch_layout(e->ls).dense, 0, dense_bytes(e->ls), st));
        if (e->ls.pair_on)
            GPM_CK(cudaMemsetAsync((char*)e->scratch + scratch_layout(e->ls).tables, 0, pair_region_bytes(e->ls), st));
    }
    e->dense_dirty = true;
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
    e->dense_dirty = false;
    return finish_counts(n, e->plans.data(), raw.data(), outs);
}

GPM_API int gpm_batch_exec_destroy(gpm_batch_exec* exec) {
    delete exec;
    return GPM_OK;
}

// ---------------------------------------------------------------------------
// Counting without any device allocation.
//
// Some callers cannot call cudaMalloc: programs whose device memory is
// reserved by another allocator (a framework's caching allocator or a fixed
// arena that owns the GPU, so a cudaMalloc fails or fragments its pool), and
// latency-critical loops that cannot afford cudaMalloc/cudaFree's implicit
// device synchronisation.  gpm_count_noalloc serves them with the scratch below: a
// file-scope device array that every GPU loading this library holds until
// the process exits.  Host code cannot use the array's name as an address;
// the device address comes from cudaGetSymbolAddress, once per device.

namespace gpm {

constexpr size_t kNoAllocBytes = 64ull << 20;  // 64 MiB
constexpr size_t kNoAllocHeader = 8192;        // control words, pair, plan
static_assert(512 + sizeof(DevPlan) <= kNoAllocHeader, "plan does not fit the header");
static_assert(sizeof(PairDesc) <= 256, "pair does not fit the header");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static void* g_noalloc_addr[64] = {nullptr};
static std::mutex g_noalloc_mu;

__global__ void max_degree_kernel(const unsigned* __restrict__ rowptr, int v_cnt, unsigned* __restrict__ out) {
    unsigned m = 0;
    for (long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x; v < v_cnt; v += (long long)gridDim.x * blockDim.x)
        m = max(m, rowptr[v + 1] - rowptr[v]);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) m = max(m, __shfl_xor_sync(kFull, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace gpm

GPM_API int gpm_count_noalloc(int32_t v_cnt, const uint32_t* d_rowptr, const int32_t* d_col, const int64_t* tables,
                              int32_t n_words, gpm_u128* out) {
    clear_error();
    if (v_cnt < 1 || !d_rowptr || !d_col || !tables || !out) {
        set_error("gpm_count_noalloc: need v_cnt >= 1, device CSR pointers, tables and out");
        return GPM_ERR_INVALID_ARG;
    }
    DevPlan hp;
    int rc = compile_plan(tables, n_words, &hp);
    if (rc) return rc;
    int dev = 0, sms = 0;
    GPM_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("gpm_count_noalloc: device %d out of range", dev);
        return GPM_ERR_NO_DEVICE;
    }
    GPM_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    unsigned char* base = nullptr;
    {
        // set-up once per device, with that device current
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_error("gpm_count_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
                return GPM_ERR_CUDA;
            }
            g_noalloc_addr[dev] = p;
        }
        base = (unsigned char*)g_noalloc_addr[dev];
    }
    cudaStream_t st = cudaStreamPerThread;
    // control words: [0] work cursor, [1..2] 128-bit sum, [3..4] stats,
    // [5..6] stripes/stripe, [7] max degree, [8..12] CSR check words
    unsigned long long* ctrl = (unsigned long long*)base;
    PairDesc* d_pair = (PairDesc*)(base + 256);
    DevPlan* d_plan = (DevPlan*)(base + 512);
    DonationArea* don = (DonationArea*)(base + kNoAllocHeader);
    const size_t don_bytes = (sizeof(DonationArea) + 255) & ~(size_t)255;
    int* warp_scratch = (int*)(base + kNoAllocHeader + don_bytes);
    const size_t scratch_room = kNoAllocBytes - kNoAllocHeader - don_bytes;
    uint32_t e_cnt = 0;
    GPM_CK(cudaMemcpyAsync(&e_cnt, d_rowptr + v_cnt, sizeof e_cnt, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    // the caller's CSR gets the checks gpm_graph_create applies
    GraphView view;
    view.rowptr = d_rowptr;
    view.col = d_col;
    view.v_cnt = v_cnt;
    view.pad_ = 0;
    view.e_cnt = e_cnt;
    const unsigned long long init[13] = {0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0};
    GPM_CK(cudaMemcpyAsync(ctrl, init, sizeof init, cudaMemcpyHostToDevice, st));
    max_degree_kernel<<<sms * 4, 256, 0, st>>>(d_rowptr, v_cnt, (unsigned*)(ctrl + 7));
    GPM_CK(cudaGetLastError());
    validate_kernel<<<sms * 8, 256, 0, st>>>(view, ctrl + 8);
    GPM_CK(cudaGetLastError());
    unsigned long long got[6] = {0, 0, 0, 0, 0, 0};
    GPM_CK(cudaMemcpyAsync(got, ctrl + 7, sizeof got, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    const unsigned maxdeg = (unsigned)got[0], flags = csr_flags(got + 1);
    if (flags) {
        set_error("gpm_count_noalloc: malformed CSR (%s%s%s%s%s)", flags & 1 ? "offsets " : "",
                  flags & 2 ? "ids-out-of-range " : "", flags & 4 ? "self-loops " : "",
                  flags & 8 ? "unsorted-or-duplicate " : "", flags & 16 ? "asymmetric" : "");
        return GPM_ERR_INVALID_ARG;
    }
    // size the grid to what the array holds and to what is resident at once
    // (idle warps help with published loops until every warp is done)
    const Options& o = options();
    const int wpb = (int)o.warps_per_block;
    const int stage_cap = o.leaf_batch ? (int)o.stage_max : 0;
    const size_t smem = sizeof(WarpState) * wpb + sizeof(int) * 2 * (size_t)stage_stride(stage_cap) * wpb;
    GPM_CK(cudaFuncSetAttribute(match_kernel<false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int occ = 0;
    GPM_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, match_kernel<false, 1>, wpb * 32, smem));
    if (occ < 1) {
        set_error("launch shape does not fit an SM: %d warps per block, %zu bytes of shared memory", wpb, smem);
        return GPM_ERR_INVALID_ARG;
    }
    const long long cap = std::max<long long>(1, maxdeg);
    const long long per_warp = (long long)hp.nslots * cap + 2 * pair_bs_stride(cap);
    const long long fit = (long long)(scratch_room / ((size_t)per_warp * sizeof(int)));
    const long long want = (long long)sms * std::min<long long>(o.blocks_per_sm, occ) * wpb;
    const long long warps = std::min(want, fit) / wpb * wpb;
    if (warps < wpb) {
        set_error("gpm_count_noalloc: one block of %d warps needs %lld bytes of scratch (%d sets x largest degree %lld "
                  "x 4 bytes per warp, and a tail of 1/16 of a set); the allocation-free scratch holds %zu bytes: use gpm_count",
                  wpb, (long long)wpb * per_warp * 4, hp.nslots, cap, scratch_room);
        return GPM_ERR_UNSUPPORTED;
    }
    PairDesc pd;
    pd.g = view;
    pd.plan = d_plan;
    pd.ntasks = hp.T == 1 ? (unsigned long long)v_cnt : (unsigned long long)e_cnt;
    pd.cap = (int)cap;
    pd.pad_ = 0;
    // grabs shrink so that no warp is left without a task (as gpm_count does)
    const int chunk = (int)std::max<long long>(1, std::min<long long>(o.chunk, (long long)(pd.ntasks / warps)));
    GPM_CK(cudaMemcpyAsync(d_pair, &pd, sizeof pd, cudaMemcpyHostToDevice, st));
    GPM_CK(cudaMemcpyAsync(d_plan, &hp, sizeof hp, cudaMemcpyHostToDevice, st));
    const int split = (int)o.split;
    if (split > 0) GPM_CK(cudaMemsetAsync(don, 0, sizeof(DonationArea), st));
    const int alpha4[3] = {(int)o.merge_alpha4[0], (int)o.merge_alpha4[1], (int)o.merge_alpha4[2]};
    GPM_CK(cudaMemcpyToSymbolAsync(c_merge_alpha4, alpha4, sizeof alpha4, 0, cudaMemcpyHostToDevice, st));
    match_kernel<false, 1><<<(unsigned)(warps / wpb), wpb * 32, smem, st>>>(
        d_pair, 1, ctrl, ctrl + 1, warp_scratch, per_warp, chunk, ctrl + 5, (int)o.leaf_batch, stage_cap,
        0, nullptr, 0, split > 0 ? don : nullptr, split, nullptr, 0, 0, nullptr, 0, 0, ctrl + 3);
    GPM_CK(cudaGetLastError());
    unsigned long long raw[2] = {0, 0};
    GPM_CK(cudaMemcpyAsync(raw, ctrl + 1, sizeof raw, cudaMemcpyDeviceToHost, st));
    GPM_CK(cudaStreamSynchronize(st));
    rc = take_check("gpm_count_noalloc");
    if (rc) return rc;
    const unsigned __int128 u = ((unsigned __int128)raw[1] << 64) | raw[0];
    if ((__int128)u < 0) {
        set_error("gpm_count_noalloc: negative total (128-bit overflow)");
        return GPM_ERR_OVERFLOW;
    }
    const unsigned __int128 q = u / (unsigned __int128)hp.redundancy;
    out->lo = (uint64_t)q;
    out->hi = (uint64_t)(q >> 64);
    return GPM_OK;
}

GPM_API int gpm_last_launch_stats(double* kernel_ms, int64_t* launches, uint64_t* algo_bytes) {
    if (kernel_ms) *kernel_ms = t_ms;
    if (launches) *launches = t_launches;
    if (algo_bytes) *algo_bytes = t_bytes;
    return GPM_OK;
}

}  // extern "C"
