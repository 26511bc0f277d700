// Row search over a CSR's offsets, shared by the edge-parallel upload
// kernels (validation, relabel fill) of gpm_device.cu; the warp emulator
// compiles it too (tests/emu).  Included inside namespace gpm after
// match_core.cuh (kFull).
#pragma once

// Row of position k of a CSR: the last r in [0, V) with rowptr[r] <= k
// (a binary search over the offsets; k < rowptr[V]).
__device__ int csr_row_of(const unsigned* __restrict__ rowptr, int V, unsigned long long k) {
    int lo = 0, hi = V - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((unsigned long long)rowptr[mid] <= k) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Rows of the 32 positions kb + lane (those below end): r0 is a row that
// starts at or before kb.  Each round, lane j holds the start of row
// r0 + 1 + j and every position finds how many of those starts it has
// passed with a 5-step shuffle search; positions past all 32 move r0 on by
// 32 rows and search again (rows of degree 0 are passed 32 at a time).
// Returns this lane's row and leaves r0 at the batch's last row.
__device__ int csr_batch_row(const unsigned* __restrict__ rowptr, int V, unsigned long long kb,
                             unsigned long long end, int& r0, int lane) {
    const unsigned long long k = kb + (unsigned long long)lane;
    int row = r0;
    bool done = k >= end;
    int base = r0;
    for (int round = 0; round < (1 << 26); ++round) {
        if (__all_sync(kFull, done)) break;
        const int r = base + 1 + lane;
        const unsigned long long start = r < V ? (unsigned long long)rowptr[r] : ~0ull;
        int c = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const unsigned long long sq = __shfl_sync(kFull, start, c + step - 1);
            if (sq <= k) c += step;
        }
        const unsigned long long s31 = __shfl_sync(kFull, start, 31);
        if (!done) {
            if (c == 31 && s31 <= k) {
                row = base + 32;  // at least: search on from there
            } else {
                row = base + c;
                done = true;
            }
        }
        base += 32;
    }
    // the batch's last row: the largest row of the lanes below end
    int last = k < end ? row : -1;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) last = max(last, __shfl_xor_sync(kFull, last, o));
    if (last >= 0) r0 = last;
    return row;
}
