// Schedule construction on the GPU: the exhaustive cost evaluation of the
// Schedule constructor (reference src/schedule.cpp:9-150) — every (loop
// order, restriction set) candidate scored by the chosen performance model
// (our_estimate_schedule_restrict :1487-1574, GraphZero_ :1576-1640,
// Naive_ :1642-1713) — one thread per candidate.
//
// The choice must equal the host's word for word, so every floating-point
// operation is an explicitly rounded intrinsic (__dadd_rn, __dmul_rn,
// __ddiv_rn: no fused multiply-add) in the host code's order, and the
// restriction ratios are recomputed per candidate by the same permutation
// walk (the fraction of the n! orders of the pattern's vertices that satisfy
// each restriction given the earlier ones).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "gpm_internal.h"

namespace gpm {

namespace {

constexpr int kSMaxN = 8;
constexpr int kSMaxPairs = 28;

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

// std::next_permutation on t[0, n)
__device__ bool next_perm(int* t, int n) {
    int i = n - 2;
    while (i >= 0 && t[i] >= t[i + 1]) --i;
    if (i < 0) return false;
    int j = n - 1;
    while (t[j] <= t[i]) --j;
    int x = t[i];
    t[i] = t[j];
    t[j] = x;
    for (int a = i + 1, b = n - 1; a < b; ++a, --b) {
        x = t[a];
        t[a] = t[b];
        t[b] = x;
    }
    return true;
}

// ratio[i] = P(restriction i holds | restrictions 0..i-1 hold), pairs sorted
__device__ void ratios(int n, const int* pr, int r, double* out) {
    for (int i = 0; i < r; ++i) out[i] = 0.0;
    int t[kSMaxN];
    for (int i = 0; i < n; ++i) t[i] = i;
    do {
        for (int i = 0; i < r; ++i) {
            if (t[pr[2 * i]] > t[pr[2 * i + 1]]) out[i] = dadd(out[i], 1.0);
            else break;
        }
    } while (next_perm(t, n));
    double total = 1;
    for (int i = 2; i <= n; ++i) total = dmul(total, (double)i);
    for (int i = 0; i < r; ++i) out[i] = ddiv(out[i], total);
    for (int i = r - 1; i > 0; --i) out[i] = ddiv(out[i], out[i - 1]);
}

// cur: the pattern in the candidate's loop order (n x n); pr: its sorted
// restriction pairs.  perf 1: our_estimate, 2: GraphZero, 3: Naive.
__global__ void score_kernel(int n, int perf, int md, const int* __restrict__ mats, const int* __restrict__ cand_order,
                             const int* __restrict__ npairs, const int* __restrict__ pairs, int count, double v,
                             double e, double tri, double* __restrict__ out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    const int* cur = mats + (size_t)cand_order[c] * n * n;
    const int r = npairs[c];
    const int* pr = pairs + (size_t)c * 2 * kSMaxPairs;
    double ratio[kSMaxPairs];
    ratios(n, pr, r, ratio);
    // invariant[j]: the values pushed while later vertices were processed
    int inv[kSMaxN][kSMaxN];
    int ninv[kSMaxN];
    for (int i = 0; i < n; ++i) ninv[i] = 0;
    double val = 1;
    if (perf == 3) {
        const double p = ddiv(ddiv(dmul(e, 2.0), v), v);
        for (int i = n - 1; i >= 0; --i) {
            int forward = 0;
            for (int j = 0; j < i; ++j) forward += cur[j * n + i] ? 1 : 0;
            for (int j = 0; j < r; ++j)
                if (pr[2 * j + 1] == i) val = dmul(val, ratio[j]);
            val = dmul(val, v);
            for (int j = 0; j < i - forward; ++j) val = dmul(val, __dsub_rn(1.0, p));
            for (int j = 0; j < forward; ++j) val = dmul(val, p);
        }
        out[c] = val;
        return;
    }
    double ps[kSMaxN + 2], pps[kSMaxN + 2];
    if (perf == 1) {
        const double p0 = ddiv(ddiv(dmul(e, 1.0), v), v);
        const double p1 = ddiv(ddiv(dmul(dmul(tri, 1.0), v), e), e);
        ps[0] = v;
        for (int i = 1; i < md; ++i) ps[i] = dmul(ps[i - 1], p0);
        pps[0] = 1;
        for (int i = 1; i < md; ++i) pps[i] = dmul(pps[i - 1], p1);
    } else {
        const double p = ddiv(ddiv(dmul(e, 1.0), v), v);
        ps[0] = v;
        for (int i = 1; i < md; ++i) ps[i] = dmul(ps[i - 1], p);
    }
    for (int i = n - 1; i >= 0; --i) {
        int forward = 0;
        for (int j = 0; j < i; ++j) forward += cur[j * n + i] ? 1 : 0;
        int cc = forward;
        for (int j = i - 1; j >= 0; --j)
            if (cur[j * n + i]) inv[j][ninv[j]++] = cc--;
        for (int q = 0; q < ninv[i]; ++q) {
            const int x = inv[i][q];
            if (x > 1) {
                if (perf == 1) val = dadd(val, dadd(dmul(ps[1], pps[x - 2]), ps[1]));
                else val = dadd(val, dadd(ps[x - 1], ps[1]));
            }
        }
        if (perf == 1) val = dadd(val, 1.0);
        for (int j = 0; j < r; ++j)
            if (pr[2 * j + 1] == i) val = dmul(val, ratio[j]);
        if (perf == 1) {
            if (i) val = dmul(val, dmul(ps[1], pps[forward - 1]));
            else val = dmul(val, ps[0]);
        } else {
            val = dmul(val, ps[forward]);
        }
    }
    out[c] = val;
}

}  // namespace

int score_candidates_gpu(int n, int perf, int pattern_max_degree, const std::vector<int>& mats,
                         const std::vector<int>& cand_order, const std::vector<int>& npairs,
                         const std::vector<int>& pairs, int v_cnt, unsigned int e_cnt, long long tri_cnt,
                         std::vector<double>& vals) {
    const int count = (int)cand_order.size();
    vals.assign(count, 0.0);
    if (count == 0) return GPM_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return GPM_ERR_NO_DEVICE;
    }
    // the host models size their power tables by the pattern's largest degree
    const int md = perf == 1 ? std::max(2, pattern_max_degree) : std::max(2, pattern_max_degree) + 1;
    if (n > kSMaxN || md > kSMaxN + 2) return GPM_ERR_UNSUPPORTED;
    int *d_mats = nullptr, *d_ord = nullptr, *d_np = nullptr, *d_pairs = nullptr;
    double* d_out = nullptr;
    int rc = GPM_OK;
    auto ok = [&](cudaError_t e) {
        if (e != cudaSuccess && rc == GPM_OK) {
            set_error("schedule scoring on the GPU: %s", cudaGetErrorString(e));
            rc = GPM_ERR_CUDA;
        }
        return rc == GPM_OK;
    };
    if (ok(cudaMalloc(&d_mats, sizeof(int) * mats.size())) && ok(cudaMalloc(&d_ord, sizeof(int) * count)) &&
        ok(cudaMalloc(&d_np, sizeof(int) * count)) && ok(cudaMalloc(&d_pairs, sizeof(int) * pairs.size())) &&
        ok(cudaMalloc(&d_out, sizeof(double) * count)) &&
        ok(cudaMemcpy(d_mats, mats.data(), sizeof(int) * mats.size(), cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_ord, cand_order.data(), sizeof(int) * count, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_np, npairs.data(), sizeof(int) * count, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_pairs, pairs.data(), sizeof(int) * pairs.size(), cudaMemcpyHostToDevice))) {
        score_kernel<<<(count + 127) / 128, 128>>>(n, perf, md, d_mats, d_ord, d_np, d_pairs, count, (double)v_cnt,
                                                   (double)e_cnt, (double)tri_cnt, d_out);
        if (ok(cudaGetLastError())) ok(cudaMemcpy(vals.data(), d_out, sizeof(double) * count, cudaMemcpyDeviceToHost));
    }
    cudaFree(d_mats);
    cudaFree(d_ord);
    cudaFree(d_np);
    cudaFree(d_pairs);
    cudaFree(d_out);
    return rc;
}

}  // namespace gpm
