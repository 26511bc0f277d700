// Seeded graph generators and host CSR utilities (include/gpm_gen.h).
// Random numbers are counter-based (SplitMix64 of seed, draw index and
// level), so the output does not depend on the thread count.
#include <parallel/algorithm>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "gpm_gen.h"
#include "gpm_internal.h"

namespace {

inline uint64_t splitmix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double uniform(uint64_t seed, uint64_t i, uint64_t j) {
    uint64_t r = splitmix(splitmix(seed ^ (i * 0xD6E8FEB86659FD93ull)) + j * 0xA0761D6478BD642Full);
    return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

// undirected (u, v) keys -> symmetric sorted deduplicated CSR
int build_csr(int32_t n, std::vector<uint64_t>& keys, uint32_t** rowptr, int32_t** col) {
    __gnu_parallel::sort(keys.begin(), keys.end());
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    if (keys.size() >= (1ull << 32)) {
        gpm::set_error("graph has %zu directed edges; the CSR offsets are 32-bit", keys.size());
        return GPM_ERR_UNSUPPORTED;
    }
    uint32_t* rp = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    int32_t* cl = (int32_t*)malloc(sizeof(int32_t) * std::max<size_t>(keys.size(), 1));
    if (!rp || !cl) {
        free(rp);
        free(cl);
        gpm::set_error("out of host memory");
        return GPM_ERR_OOM;
    }
    std::vector<uint32_t> deg((size_t)n + 1, 0);
    for (uint64_t k : keys) ++deg[k >> 32];
    rp[0] = 0;
    for (int32_t v = 0; v < n; ++v) rp[v + 1] = rp[v] + deg[v];
    const int64_t m = (int64_t)keys.size();
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < m; ++i) cl[i] = (int32_t)(keys[i] & 0xffffffffu);
    *rowptr = rp;
    *col = cl;
    return GPM_OK;
}

inline void push_undirected(std::vector<uint64_t>& keys, size_t at, uint32_t u, uint32_t v) {
    keys[at] = ((uint64_t)u << 32) | v;
    keys[at + 1] = ((uint64_t)v << 32) | u;
}

}  // namespace

extern "C" {

GPM_API void gpm_free(void* p) { free(p); }

GPM_API int gpm_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                         uint32_t** rowptr, int32_t** col, int32_t* v_cnt) {
    gpm::clear_error();
    if (scale < 1 || scale > 30 || edge_factor < 1 || !rowptr || !col || !v_cnt || a < 0 || b < 0 || c < 0 ||
        a + b + c > 1) {
        gpm::set_error("gpm_gen_rmat: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    const int32_t n = 1 << scale;
    const int64_t draws = (int64_t)edge_factor << scale;
    std::vector<uint64_t> keys((size_t)draws * 2);
    std::vector<char> keep((size_t)draws);
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < draws; ++i) {
        uint32_t u = 0, v = 0;
        for (int l = 0; l < scale; ++l) {
            const double r = uniform(seed, (uint64_t)i, (uint64_t)l);
            const uint32_t bu = r >= ab, bv = (r >= a && r < ab) || r >= abc;
            u = (u << 1) | bu;
            v = (v << 1) | bv;
        }
        keep[i] = u != v;
        push_undirected(keys, 2 * (size_t)i, u, v);
    }
    size_t w = 0;
    for (int64_t i = 0; i < draws; ++i)
        if (keep[i]) {
            keys[w] = keys[2 * i];
            keys[w + 1] = keys[2 * i + 1];
            w += 2;
        }
    keys.resize(w);
    *v_cnt = n;
    return build_csr(n, keys, rowptr, col);
}

GPM_API int gpm_gen_chung_lu(int32_t n, double avg_degree, double gamma, int32_t max_degree, uint64_t seed,
                             uint32_t** rowptr, int32_t** col, int32_t* v_cnt) {
    gpm::clear_error();
    if (n < 2 || avg_degree <= 0 || gamma <= 1.0 || !rowptr || !col || !v_cnt) {
        gpm::set_error("gpm_gen_chung_lu: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    std::vector<double> w(n);
    for (int32_t i = 0; i < n; ++i) w[i] = std::pow((double)(i + 1), -1.0 / (gamma - 1.0));
    const double target = (double)n * avg_degree;
    // scale to the target mass, capping weights at max_degree
    for (int it = 0; it < 50; ++it) {
        double s = 0;
        for (double x : w) s += x;
        const double f = target / s;
        bool changed = false;
        for (double& x : w) {
            x *= f;
            if (max_degree > 0 && x > max_degree) {
                x = max_degree;
                changed = true;
            }
        }
        if (!changed && std::fabs(f - 1.0) < 1e-12) break;
    }
    std::vector<double> cdf(n);
    std::partial_sum(w.begin(), w.end(), cdf.begin());
    const double total = cdf.back();
    const int64_t draws = (int64_t)std::llround(target / 2.0);
    std::vector<uint64_t> keys((size_t)draws * 2);
    std::vector<char> keep((size_t)draws);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < draws; ++i) {
        const double r1 = uniform(seed, (uint64_t)i, 0) * total, r2 = uniform(seed, (uint64_t)i, 1) * total;
        uint32_t u = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r1) - cdf.begin());
        uint32_t v = (uint32_t)(std::upper_bound(cdf.begin(), cdf.end(), r2) - cdf.begin());
        if (u >= (uint32_t)n) u = n - 1;
        if (v >= (uint32_t)n) v = n - 1;
        keep[i] = u != v;
        push_undirected(keys, 2 * (size_t)i, u, v);
    }
    size_t wr = 0;
    for (int64_t i = 0; i < draws; ++i)
        if (keep[i]) {
            keys[wr] = keys[2 * i];
            keys[wr + 1] = keys[2 * i + 1];
            wr += 2;
        }
    keys.resize(wr);
    *v_cnt = n;
    return build_csr(n, keys, rowptr, col);
}

GPM_API int gpm_csr_from_edges(int32_t v_cnt, int64_t m, const int32_t* src, const int32_t* dst, uint32_t** rowptr,
                               int32_t** col) {
    gpm::clear_error();
    if (v_cnt < 1 || m < 0 || (m > 0 && (!src || !dst)) || !rowptr || !col) {
        gpm::set_error("gpm_csr_from_edges: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    std::vector<uint64_t> keys;
    keys.reserve((size_t)m * 2);
    for (int64_t i = 0; i < m; ++i) {
        if (src[i] < 0 || src[i] >= v_cnt || dst[i] < 0 || dst[i] >= v_cnt) {
            gpm::set_error("gpm_csr_from_edges: edge %lld has an endpoint outside [0, %d)", (long long)i, v_cnt);
            return GPM_ERR_INVALID_ARG;
        }
        if (src[i] == dst[i]) continue;
        keys.push_back(((uint64_t)(uint32_t)src[i] << 32) | (uint32_t)dst[i]);
        keys.push_back(((uint64_t)(uint32_t)dst[i] << 32) | (uint32_t)src[i]);
    }
    return build_csr(v_cnt, keys, rowptr, col);
}

GPM_API int gpm_csr_relabel_degree(int32_t n, const uint32_t* rowptr, const int32_t* col, uint32_t** rowptr_out,
                                   int32_t** col_out) {
    gpm::clear_error();
    if (n < 1 || !rowptr || !col || !rowptr_out || !col_out) {
        gpm::set_error("gpm_csr_relabel_degree: bad arguments");
        return GPM_ERR_INVALID_ARG;
    }
    std::vector<int32_t> order(n), new_id(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return rowptr[x + 1] - rowptr[x] > rowptr[y + 1] - rowptr[y];
    });
    for (int32_t i = 0; i < n; ++i) new_id[order[i]] = i;
    const uint32_t m = rowptr[n];
    uint32_t* rp = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    int32_t* cl = (int32_t*)malloc(sizeof(int32_t) * std::max<size_t>(m, 1));
    if (!rp || !cl) {
        free(rp);
        free(cl);
        gpm::set_error("out of host memory");
        return GPM_ERR_OOM;
    }
    rp[0] = 0;
    for (int32_t i = 0; i < n; ++i) rp[i + 1] = rp[i] + (rowptr[order[i] + 1] - rowptr[order[i]]);
#pragma omp parallel for schedule(dynamic, 1024)
    for (int32_t i = 0; i < n; ++i) {
        const int32_t o = order[i];
        int32_t* out = cl + rp[i];
        for (uint32_t k = rowptr[o]; k < rowptr[o + 1]; ++k) *out++ = new_id[col[k]];
        std::sort(cl + rp[i], cl + rp[i + 1]);
    }
    *rowptr_out = rp;
    *col_out = cl;
    return GPM_OK;
}

}  // extern "C"
