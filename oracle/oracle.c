/*
 * oracle.c — CPU oracle for the GB300 pattern matcher.  TEST INFRASTRUCTURE
 * ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it as the checker; the product never links, loads or calls it.
 *
 * It restates, in plain C with OpenMP, the reference GraphPi single-node
 * counting path so GPU results can be compared bit for bit:
 *   oracle_pattern_matching  Graph::pattern_matching + ..._aggressive_func
 *                            (src/graph.cpp:199-398), VertexSet::intersection
 *                            (src/vertex_set.cpp:56-120), intersection_with
 *                            (:122-156), build_vertex_set (:158-170),
 *                            has_data (:188-194), unorderd_subtraction_size
 *                            (:196-209).  Sums are 128-bit where the
 *                            reference's long long would overflow.
 *   oracle_stripes_raw       the same counting split into the GPU engine's
 *                            first-level tasks (root vertices or directed
 *                            edges), summed per stripe t mod S == s: the
 *                            root loop (src/graph.cpp:212-228) and one
 *                            depth-1 iteration (:366-396) per task
 *   oracle_pattern_matching_clique
 *                            the same with the clique function
 *                            (pattern_matching_func, src/graph.cpp:147-197,
 *                            clipped intersection src/vertex_set.cpp:75-103)
 *   oracle_triangle_count    Graph::triangle_counting_mt / tc_mt
 *                            (src/graph.cpp:66-95, 112-139)
 *   oracle_brute_force       an independent definition-level count:
 *                            injective maps preserving pattern edges, divided
 *                            by the automorphism count (no schedule at all).
 * Schedules arrive as the int64 tables of gpm_schedule_build (include/gpm.h),
 * which tests pin against the reference's own Schedule separately.
 */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef __int128 i128;

#define MAXN 8
#define MAXP 28
#define MAXG 1024
#define MAXE 4096

typedef struct {
    int n, P, R, k, ngroups;
    int father[MAXP], last[MAXN], next[MAXP], loop_set[MAXN];
    int rlast[MAXN], rnext[MAXP], rindex[MAXP];
    long long coef[MAXG];
    int gbeg[MAXG + 1]; /* blocks of group g: [gbeg[g], gbeg[g+1]) */
    int bbeg[MAXE + 1]; /* members of block b: bmem[bbeg[b] .. bbeg[b+1]) */
    int bmem[MAXE];
    long long redundancy;
} sched_t;

static int parse(const int64_t* t, int nw, sched_t* s) {
    int pos = 0;
#define GET() (pos < nw ? t[pos++] : (pos = nw + 1, 0))
    memset(s, 0, sizeof *s);
    s->n = (int)GET();
    if (s->n < 2 || s->n > MAXN) return -1;
    for (int i = 0; i < s->n * s->n; ++i) GET();
    s->P = (int)GET();
    if (s->P < 1 || s->P > MAXP) return -1;
    for (int i = 0; i < s->P; ++i) s->father[i] = (int)GET();
    for (int i = 0; i < s->n; ++i) s->last[i] = (int)GET();
    for (int i = 0; i < s->P; ++i) s->next[i] = (int)GET();
    for (int i = 0; i < s->n; ++i) s->loop_set[i] = (int)GET();
    s->R = (int)GET();
    if (s->R < 0 || s->R > MAXP) return -1;
    for (int i = 0; i < s->n; ++i) s->rlast[i] = (int)GET();
    for (int i = 0; i < s->R; ++i) s->rnext[i] = (int)GET();
    for (int i = 0; i < s->R; ++i) s->rindex[i] = (int)GET();
    int np = (int)GET();
    for (int i = 0; i < 2 * np; ++i) GET();
    s->k = (int)GET();
    s->ngroups = (int)GET();
    if (s->ngroups < 0 || s->ngroups > MAXG) return -1;
    int nb = 0, nm = 0;
    for (int g = 0; g < s->ngroups; ++g) {
        s->coef[g] = GET();
        s->gbeg[g] = nb;
        int blocks = (int)GET();
        for (int b = 0; b < blocks; ++b) {
            if (nb >= MAXE) return -1;
            int len = (int)GET();
            s->bbeg[nb] = nm;
            for (int j = 0; j < len; ++j) {
                if (nm >= MAXE) return -1;
                s->bmem[nm++] = (int)GET();
            }
            ++nb;
        }
    }
    s->gbeg[s->ngroups] = nb;
    s->bbeg[nb] = nm;
    s->redundancy = GET();
    if (pos > nw || s->redundancy < 1) return -1;
#undef GET
    return 0;
}

typedef struct {
    const uint32_t* rp;
    const int32_t* col;
    int V;
    const sched_t* s;
    int cap;
    double deadline;   /* omp_get_wtime() limit; 0: none */
    long long calls;
    int expired;
    int* buf[MAXP];
    const int* ptr[MAXP];
    int len[MAXP];
    int chosen[MAXN];
    int nchosen;
    int* tmp;
    int* tmp2;
    i128 ans;
} ctx_t;

/* merge intersection (src/vertex_set.cpp:105-119) */
static int merge(const int* a, int na, const int* b, int nb, int* out) {
    int i = 0, j = 0, w = 0;
    while (i < na && j < nb) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else {
            out[w++] = a[i];
            ++i;
            ++j;
        }
    }
    return w;
}

static int lower_bound_i(const int* a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int m = (lo + hi) >> 1;
        if (a[m] < x) lo = m + 1;
        else hi = m;
    }
    return lo;
}

/* |S[0, len) \ chosen| by binary search of each chosen vertex */
static long long outside(const ctx_t* c, const int* S, int len) {
    long long r = len;
    for (int j = 0; j < c->nchosen; ++j) {
        int p = lower_bound_i(S, len, c->chosen[j]);
        if (p < len && S[p] == c->chosen[j]) --r;
    }
    return r;
}

static void build(ctx_t* c, int pid, int v) {
    const int* nv = c->col + c->rp[v];
    int dv = (int)(c->rp[v + 1] - c->rp[v]);
    int f = c->s->father[pid];
    if (f == -1) {
        c->ptr[pid] = nv;
        c->len[pid] = dv;
        return;
    }
    /* intersection() of a set with itself copies it (src/vertex_set.cpp:58) */
    c->len[pid] = merge(c->ptr[f], c->len[f], nv, dv, c->buf[pid]);
    c->ptr[pid] = c->buf[pid];
}

static int bound_at(const ctx_t* c, int depth) {
    int mv = c->V;
    for (int i = c->s->rlast[depth]; i != -1; i = c->s->rnext[i]) {
        int x = c->chosen[c->s->rindex[i]];
        if (mv > x) mv = x;
    }
    return mv;
}

static void rec_range(ctx_t* c, int depth, int lo, int hi);
static void rec(ctx_t* c, int depth) { rec_range(c, depth, 0, 0x7fffffff); }

/* The recursion at `depth`; a loop level runs only its candidates [lo, hi)
 * (a part of the loop, so that one long loop can be shared by threads). */
static void rec_range(ctx_t* c, int depth, int lo, int hi) {
    const sched_t* s = c->s;
    if (c->deadline > 0 && (++c->calls & 1023) == 0 && omp_get_wtime() > c->deadline) c->expired = 1;
    if (c->expired) return;
    int lsid = s->loop_set[depth];
    const int* S = c->ptr[lsid];
    int size = c->len[lsid];
    if (size <= 0) return;
    if (depth == s->n - s->k) { /* inclusion–exclusion tail, src/graph.cpp:306-344 */
        for (int g = 0; g < s->ngroups; ++g) {
            i128 val = s->coef[g];
            for (int b = s->gbeg[g]; b < s->gbeg[g + 1]; ++b) {
                int m0 = s->bmem[s->bbeg[b]];
                int cnt = s->bbeg[b + 1] - s->bbeg[b];
                const int* A = c->ptr[s->loop_set[depth + m0]];
                int na = c->len[s->loop_set[depth + m0]];
                if (cnt == 1) {
                    val *= outside(c, A, na);
                } else {
                    int* dst = c->tmp;
                    for (int q = 1; q < cnt; ++q) {
                        int id = s->loop_set[depth + s->bmem[s->bbeg[b] + q]];
                        na = merge(A, na, c->ptr[id], c->len[id], dst);
                        A = dst;
                        dst = (dst == c->tmp) ? c->tmp2 : c->tmp;
                    }
                    val *= outside(c, A, na);
                }
                if (val == 0) break;
            }
            c->ans += val;
        }
        return;
    }
    if (depth == s->n - 1) { /* src/graph.cpp:346-364 */
        if (s->R > 0) {
            int lb = lower_bound_i(S, size, bound_at(c, depth));
            if (lb > 0) c->ans += outside(c, S, lb);
        } else {
            c->ans += outside(c, S, size);
        }
        return;
    }
    int mv = bound_at(c, depth); /* src/graph.cpp:367-396 */
    if (hi > size) hi = size;
    for (int i = lo; i < hi; ++i) {
        int v = S[i];
        if (mv <= v) break;
        int dup = 0;
        for (int j = 0; j < c->nchosen; ++j) dup |= c->chosen[j] == v;
        if (dup) continue;
        int zero = 0;
        for (int p = s->last[depth]; p != -1; p = s->next[p]) {
            build(c, p, v);
            if (c->len[p] == 0) {
                zero = 1;
                break;
            }
        }
        if (zero) continue;
        c->chosen[c->nchosen++] = v;
        rec(c, depth + 1);
        --c->nchosen;
    }
}

static int max_isect(int V, const uint32_t* rp) {
    int m1 = 0, m2 = 0;
    for (int v = 0; v < V; ++v) {
        int d = (int)(rp[v + 1] - rp[v]);
        if (d > m1) {
            m2 = m1;
            m1 = d;
        } else if (d > m2) {
            m2 = d;
        }
    }
    return m1 > 0 ? m1 : 1; /* largest degree bounds every set we build */
}

/* Raw sum over the roots in `roots` (all roots when roots == NULL) before the
 * division by the redundancy; out = {lo, hi} two's complement. */
static int run(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw, const int32_t* roots,
               int64_t nroots, int threads, double seconds, int64_t* done, uint64_t* out) {
    sched_t s;
    if (parse(tables, nw, &s)) return -1;
    int cap = max_isect(V, rp);
    int64_t total = roots ? nroots : V;
    i128 sum = 0;
    int bad = 0;
    int64_t completed = 0;
    const double deadline = seconds > 0 ? omp_get_wtime() + seconds : 0;
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads()) reduction(| : bad)
    {
        ctx_t c;
        memset(&c, 0, sizeof c);
        c.rp = rp;
        c.col = col;
        c.V = V;
        c.s = &s;
        c.cap = cap;
        c.deadline = deadline;
        int64_t my_done = 0;
        for (int p = 0; p < s.P; ++p) {
            c.buf[p] = (int*)malloc(sizeof(int) * (size_t)cap);
            if (!c.buf[p]) bad = 1;
        }
        c.tmp = (int*)malloc(sizeof(int) * (size_t)cap);
        c.tmp2 = (int*)malloc(sizeof(int) * (size_t)cap);
        if (!c.tmp || !c.tmp2) bad = 1;
        if (!bad) {
#pragma omp for schedule(dynamic, 16)
            for (int64_t r = 0; r < total; ++r) {
                if (c.expired) continue;
                int v = roots ? roots[r] : (int)r;
                i128 before = c.ans;
                for (int p = s.last[0]; p != -1; p = s.next[p]) build(&c, p, v);
                c.nchosen = 0;
                c.chosen[c.nchosen++] = v;
                rec(&c, 1);
                if (c.expired) c.ans = before; /* drop the unfinished root */
                else ++my_done;
            }
        }
#pragma omp critical
        {
            sum += c.ans;
            completed += my_done;
        }
        for (int p = 0; p < s.P; ++p) free(c.buf[p]);
        free(c.tmp);
        free(c.tmp2);
    }
    if (bad) return -2;
    if (done) *done = completed;
    out[0] = (uint64_t)sum;
    out[1] = (uint64_t)(sum >> 64);
    return 0;
}

int oracle_pattern_matching(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw, int threads,
                            uint64_t* out) {
    uint64_t raw[2];
    sched_t s;
    if (parse(tables, nw, &s)) return -1;
    int rc = run(V, rp, col, tables, nw, NULL, 0, threads, 0, NULL, raw);
    if (rc) return rc;
    i128 sum = (i128)(((unsigned __int128)raw[1] << 64) | raw[0]);
    if (sum < 0) return -3;
    unsigned __int128 q = (unsigned __int128)sum / (unsigned __int128)s.redundancy;
    out[0] = (uint64_t)q;
    out[1] = (uint64_t)(q >> 64);
    return 0;
}

int oracle_pattern_matching_roots(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw,
                                  const int32_t* roots, int64_t nroots, int threads, uint64_t* raw) {
    return run(V, rp, col, tables, nw, roots, nroots, threads, 0, NULL, raw);
}

/* As above, but stops after `seconds` of wall time: roots not finished by
 * then are left out; *done receives how many roots were counted in full. */
int oracle_pattern_matching_roots_timed(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw,
                                        const int32_t* roots, int64_t nroots, int threads, double seconds,
                                        int64_t* done, uint64_t* raw) {
    return run(V, rp, col, tables, nw, roots, nroots, threads, seconds, done, raw);
}

/* ---- the clique path ------------------------------------------------------
 *
 * Graph::pattern_matching_func with clique = true (src/graph.cpp:147-197):
 * no restrictions and no injectivity checks; a loop stops at the first
 * candidate not below the last chosen vertex, every prefix set with a father
 * keeps only the elements below the vertex just chosen
 * (VertexSet::intersection's min_vertex clip, src/vertex_set.cpp:75-103),
 * and the last level adds its loop set's size.  For a clique pattern every
 * clique is counted once, as its decreasing vertex sequence. */
static int ctx_alloc(ctx_t* c, const uint32_t* rp, const int32_t* col, int V, int cap);
static void ctx_free(ctx_t* c);

static int merge_below(const int* a, int na, const int* b, int nb, int lim, int* out) {
    int i = 0, j = 0, w = 0;
    while (i < na && j < nb && a[i] < lim && b[j] < lim) {
        if (a[i] < b[j]) ++i;
        else if (a[i] > b[j]) ++j;
        else {
            out[w++] = a[i];
            ++i;
            ++j;
        }
    }
    return w;
}

static void clique_rec(ctx_t* c, int depth) {
    const sched_t* s = c->s;
    const int lsid = s->loop_set[depth];
    const int* S = c->ptr[lsid];
    const int size = c->len[lsid];
    if (size <= 0) return;
    if (depth == s->n - 1) {
        c->ans += size;
        return;
    }
    const int last = c->chosen[c->nchosen - 1];
    for (int i = 0; i < size; ++i) {
        const int v = S[i];
        if (last <= v) break;
        int zero = 0;
        for (int p = s->last[depth]; p != -1; p = s->next[p]) {
            const int* nv = c->col + c->rp[v];
            const int dv = (int)(c->rp[v + 1] - c->rp[v]);
            const int f = s->father[p];
            if (f == -1) {
                c->ptr[p] = nv;
                c->len[p] = dv;
            } else {
                c->len[p] = merge_below(c->ptr[f], c->len[f], nv, dv, v, c->buf[p]);
                c->ptr[p] = c->buf[p];
            }
            if (c->len[p] == 0) {
                zero = 1;
                break;
            }
        }
        if (zero) continue;
        c->chosen[c->nchosen++] = v;
        clique_rec(c, depth + 1);
        --c->nchosen;
    }
}

/* Graph::pattern_matching's root loop with the clique function, divided by
 * the redundancy (src/graph.cpp:199-245). */
int oracle_pattern_matching_clique(int V, const uint32_t* rp, const int32_t* col, const int64_t* tables, int nw,
                                   int threads, uint64_t* out) {
    sched_t s;
    if (parse(tables, nw, &s)) return -1;
    const int cap = max_isect(V, rp);
    i128 sum = 0;
    int bad = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads()) reduction(| : bad)
    {
        ctx_t c;
        if (ctx_alloc(&c, rp, col, V, cap)) bad = 1;
        c.s = &s;
        if (!bad) {
#pragma omp for schedule(dynamic, 16)
            for (int v = 0; v < V; ++v) {
                for (int p = s.last[0]; p != -1; p = s.next[p]) build(&c, p, v);
                c.nchosen = 0;
                c.chosen[c.nchosen++] = v;
                clique_rec(&c, 1);
            }
        }
#pragma omp critical
        sum += c.ans;
        ctx_free(&c);
    }
    if (bad) return -2;
    unsigned __int128 q = (unsigned __int128)sum / (unsigned __int128)s.redundancy;
    out[0] = (uint64_t)q;
    out[1] = (uint64_t)(q >> 64);
    return 0;
}

/* ---- the engine's first-level tasks, stripe by stripe --------------------
 *
 * The GPU engine splits a job into first-level tasks: root vertices when the
 * inclusion–exclusion tail starts at depth 1 (n - k == 1), otherwise the
 * directed edges e of the CSR, task e = (v0, v1) with v0 the row holding e
 * and v1 = col[e].  Stripe s of S holds the tasks t with t mod S == s.  This
 * restates, per task, the reference's root loop (src/graph.cpp:212-228: the
 * depth-0 prefix sets of v0) and one iteration of the depth-1 loop of
 * pattern_matching_aggressive_func for the candidate v1 (:366-396:
 * restriction bound, has_data, prefix sets of depth 1, empty-set skip), then
 * the recursion from depth 2 (rec above).  A root task is the reference's
 * root loop body itself.  Sums are the undivided signed 128-bit totals, so
 * stripes add up to the whole job before the division by the redundancy. */
static void task_sum(ctx_t* c, int T, int64_t t, int lo, int hi) {
    const sched_t* s = c->s;
    int v0, v1 = -1;
    if (T == 1) {
        v0 = (int)t;
    } else {
        /* last row v with rp[v] <= t */
        int lo = 0, hi = c->V;
        while (lo < hi) {
            int mid = (int)(((int64_t)lo + hi + 1) >> 1);
            if ((int64_t)c->rp[mid] <= t) lo = mid;
            else hi = mid - 1;
        }
        v0 = lo;
        v1 = c->col[t];
    }
    for (int p = s->last[0]; p != -1; p = s->next[p]) build(c, p, v0);
    c->nchosen = 0;
    c->chosen[c->nchosen++] = v0;
    if (T == 1) {
        rec(c, 1);
        return;
    }
    if (bound_at(c, 1) <= v1) return;
    if (v1 == v0) return;
    for (int p = s->last[1]; p != -1; p = s->next[p]) {
        build(c, p, v1);
        if (c->len[p] == 0) return;
    }
    c->chosen[c->nchosen++] = v1;
    rec_range(c, 2, lo, hi);
}

/* Candidates of the depth-2 loop of task t (0 when depth 2 is not a loop
 * level or the task ends earlier): the part of the loop set below the
 * restriction bound. */
static int depth2_len(ctx_t* c, int T, int64_t t) {
    const sched_t* s = c->s;
    if (T < 3 || s->n - 1 <= 2) return 0;
    int lo = 0, hi = c->V;
    while (lo < hi) {
        int mid = (int)(((int64_t)lo + hi + 1) >> 1);
        if ((int64_t)c->rp[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const int v0 = lo, v1 = c->col[t];
    for (int p = s->last[0]; p != -1; p = s->next[p]) build(c, p, v0);
    c->nchosen = 0;
    c->chosen[c->nchosen++] = v0;
    if (bound_at(c, 1) <= v1 || v1 == v0) return 0;
    for (int p = s->last[1]; p != -1; p = s->next[p]) {
        build(c, p, v1);
        if (c->len[p] == 0) return 0;
    }
    c->chosen[c->nchosen++] = v1;
    const int sid = s->loop_set[2];
    return lower_bound_i(c->ptr[sid], c->len[sid], bound_at(c, 2));
}

/* Per-thread scratch of the stripe counter. */
static int ctx_alloc(ctx_t* c, const uint32_t* rp, const int32_t* col, int V, int cap) {
    memset(c, 0, sizeof *c);
    c->rp = rp;
    c->col = col;
    c->V = V;
    c->cap = cap;
    int bad = 0;
    for (int p = 0; p < MAXP; ++p) {
        c->buf[p] = (int*)malloc(sizeof(int) * (size_t)cap);
        if (!c->buf[p]) bad = 1;
    }
    c->tmp = (int*)malloc(sizeof(int) * (size_t)cap);
    c->tmp2 = (int*)malloc(sizeof(int) * (size_t)cap);
    return bad || !c->tmp || !c->tmp2;
}

static void ctx_free(ctx_t* c) {
    for (int p = 0; p < MAXP; ++p) free(c->buf[p]);
    free(c->tmp);
    free(c->tmp2);
}

/* Raw sums of n_sched schedules (tables concatenated, nw[i] words each) over
 * the stripes ids[0, n_ids) of `stripes`: out[2*(i*n_ids + j) ..] = {lo, hi}
 * of schedule i on stripe ids[j].  All (schedule, task) pairs run in one
 * dynamically scheduled loop over the host threads; a task whose depth-2 loop
 * is long is cut into parts of kPart candidates first, so that one heavy
 * task does not run on one thread alone (the sums are the same: the loop's
 * total is the sum of its parts). */
#define kPart 8
int oracle_stripes_raw(int V, const uint32_t* rp, const int32_t* col, int n_sched, const int64_t* tables,
                       const int32_t* nw, int64_t stripes, const int64_t* ids, int n_ids, int threads, uint64_t* out) {
    if (n_sched < 1 || n_ids < 1 || stripes < 1) return -1;
    const int nth = threads > 0 ? threads : omp_get_max_threads();
    sched_t* sc = (sched_t*)calloc((size_t)n_sched, sizeof(sched_t));
    int* Ts = (int*)calloc((size_t)n_sched, sizeof(int));
    int rc = 0;
    int64_t off = 0, total = 0;
    if (!sc || !Ts) rc = -2;
    for (int i = 0; i < n_sched && !rc; ++i) {
        if (parse(tables + off, nw[i], &sc[i])) rc = -1;
        off += nw[i];
        Ts[i] = sc[i].k ? sc[i].n - sc[i].k : sc[i].n - 1;
    }
    for (int j = 0; j < n_ids && !rc; ++j)
        if (ids[j] < 0 || ids[j] >= stripes) rc = -1;
    if (rc) {
        free(sc);
        free(Ts);
        return rc;
    }
    /* tasks: (output index, task id) */
    for (int i = 0; i < n_sched; ++i) {
        const int64_t nt = Ts[i] == 1 ? (int64_t)V : (int64_t)rp[V];
        for (int j = 0; j < n_ids; ++j)
            if (ids[j] < nt) total += (nt - ids[j] + stripes - 1) / stripes;
    }
    const size_t nt1 = (size_t)(total > 0 ? total : 1);
    int32_t* ti = (int32_t*)malloc(sizeof(int32_t) * nt1);
    int64_t* tt = (int64_t*)malloc(sizeof(int64_t) * nt1);
    int32_t* tl = (int32_t*)malloc(sizeof(int32_t) * nt1); /* depth-2 loop length */
    int64_t* first = (int64_t*)malloc(sizeof(int64_t) * (nt1 + 1));
    i128* acc = (i128*)calloc((size_t)n_sched * n_ids, sizeof(i128));
    if (!ti || !tt || !tl || !first || !acc) rc = -2;
    if (!rc) {
        int64_t w = 0;
        for (int i = 0; i < n_sched; ++i) {
            const int64_t nt = Ts[i] == 1 ? (int64_t)V : (int64_t)rp[V];
            for (int j = 0; j < n_ids; ++j)
                for (int64_t t = ids[j]; t < nt; t += stripes) {
                    ti[w] = i * n_ids + j;
                    tt[w] = t;
                    ++w;
                }
        }
    }
    const int cap = max_isect(V, rp);
    int bad = rc != 0;
    /* phase 1: the length of every task's depth-2 loop */
    if (!bad) {
#pragma omp parallel num_threads(nth) reduction(| : bad)
        {
            ctx_t c;
            if (ctx_alloc(&c, rp, col, V, cap)) bad = 1;
            if (!bad) {
#pragma omp for schedule(dynamic, 16)
                for (int64_t x = 0; x < total; ++x) {
                    const int i = ti[x] / n_ids;
                    c.s = &sc[i];
                    tl[x] = depth2_len(&c, Ts[i], tt[x]);
                }
            }
            ctx_free(&c);
        }
    }
    /* work items: task x, candidates [q*kPart, q*kPart + kPart) of its loop */
    int64_t items = 0;
    if (!bad) {
        for (int64_t x = 0; x < total; ++x) {
            first[x] = items;
            items += tl[x] > kPart ? (tl[x] + kPart - 1) / kPart : 1;
        }
        first[total] = items;
    }
    if (!bad) {
#pragma omp parallel num_threads(nth) reduction(| : bad)
        {
            ctx_t c;
            if (ctx_alloc(&c, rp, col, V, cap)) bad = 1;
            i128* mine = (i128*)calloc((size_t)n_sched * n_ids, sizeof(i128));
            if (!mine) bad = 1;
            if (!bad) {
                int64_t x = 0;
#pragma omp for schedule(dynamic, 1)
                for (int64_t it = 0; it < items; ++it) {
                    /* the task holding item `it` (items are in task order) */
                    int64_t a = 0, b = total - 1;
                    while (a < b) {
                        int64_t m = (a + b + 1) >> 1;
                        if (first[m] <= it) a = m;
                        else b = m - 1;
                    }
                    x = a;
                    const int i = ti[x] / n_ids;
                    c.s = &sc[i];
                    c.ans = 0;
                    int lo = 0, hi = 0x7fffffff;
                    if (tl[x] > kPart) {
                        lo = (int)(it - first[x]) * kPart;
                        hi = lo + kPart;
                    }
                    task_sum(&c, Ts[i], tt[x], lo, hi);
                    mine[ti[x]] += c.ans;
                }
#pragma omp critical
                for (int q = 0; q < n_sched * n_ids; ++q) acc[q] += mine[q];
            }
            free(mine);
            ctx_free(&c);
        }
    }
    if (!bad)
        for (int q = 0; q < n_sched * n_ids; ++q) {
            out[2 * q] = (uint64_t)acc[q];
            out[2 * q + 1] = (uint64_t)(acc[q] >> 64);
        }
    free(sc);
    free(Ts);
    free(ti);
    free(tt);
    free(tl);
    free(first);
    free(acc);
    return bad ? (rc ? rc : -2) : 0;
}

long long oracle_triangle_count(int V, const uint32_t* rp, const int32_t* col, int threads) {
    long long total = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : total) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int v = 0; v < V; ++v) {
        for (uint32_t e = rp[v]; e < rp[v + 1]; ++e) {
            int u = col[e];
            if (v <= u) break;
            /* common neighbours of v and u below u */
            uint32_t a = rp[v], b = rp[v + 1], x = rp[u], y = rp[u + 1];
            while (a < b && x < y && col[a] < u && col[x] < u) {
                if (col[a] < col[x]) ++a;
                else if (col[x] < col[a]) ++x;
                else {
                    ++total;
                    ++a;
                    ++x;
                }
            }
        }
    }
    return total;
}

/* ---- brute force from the definition ------------------------------------ */

typedef struct {
    const uint32_t* rp;
    const int32_t* col;
    int V, n;
    int order[MAXN];        /* pattern vertices in a connected order */
    int anchor[MAXN];       /* an earlier neighbour of order[i] (i >= 1) */
    int adj[MAXN * MAXN];
    int map[MAXN];          /* pattern vertex -> graph vertex */
    i128 count;
} bf_t;

static int has_edge(const bf_t* b, int u, int v) {
    const int* a = b->col + b->rp[u];
    int d = (int)(b->rp[u + 1] - b->rp[u]);
    int p = lower_bound_i(a, d, v);
    return p < d && a[p] == v;
}

static void bf_rec(bf_t* b, int i) {
    if (i == b->n) {
        b->count += 1;
        return;
    }
    int pv = b->order[i];
    int base = b->map[b->anchor[i]];
    for (uint32_t e = b->rp[base]; e < b->rp[base + 1]; ++e) {
        int g = b->col[e];
        int ok = 1;
        for (int j = 0; j < i && ok; ++j) {
            int qv = b->order[j];
            if (b->map[qv] == g) ok = 0;
            else if (b->adj[pv * b->n + qv] && !has_edge(b, g, b->map[qv])) ok = 0;
        }
        if (!ok) continue;
        b->map[pv] = g;
        bf_rec(b, i + 1);
    }
}

/* Embeddings of the (connected) pattern: injective edge-preserving maps over
 * |Aut|.  Returns -1 for a disconnected or oversized pattern. */
int oracle_brute_force(int V, const uint32_t* rp, const int32_t* col, int n, const int32_t* adj, int threads,
                       uint64_t* out) {
    if (n < 1 || n > MAXN) return -1;
    bf_t proto;
    memset(&proto, 0, sizeof proto);
    proto.rp = rp;
    proto.col = col;
    proto.V = V;
    proto.n = n;
    for (int i = 0; i < n * n; ++i) proto.adj[i] = adj[i] != 0;
    int used[MAXN] = {0};
    proto.order[0] = 0;
    used[0] = 1;
    for (int i = 1; i < n; ++i) {
        int found = 0;
        for (int v = 0; v < n && !found; ++v) {
            if (used[v]) continue;
            for (int j = 0; j < i; ++j)
                if (proto.adj[v * n + proto.order[j]]) {
                    proto.order[i] = v;
                    proto.anchor[i] = proto.order[j];
                    used[v] = 1;
                    found = 1;
                    break;
                }
        }
        if (!found) return -1;
    }
    /* automorphisms of the pattern */
    long long aut = 0;
    {
        int p[MAXN];
        for (int i = 0; i < n; ++i) p[i] = i;
        for (;;) {
            int ok = 1;
            for (int i = 0; i < n && ok; ++i)
                for (int j = 0; j < n; ++j)
                    if (proto.adj[i * n + j] != proto.adj[p[i] * n + p[j]]) {
                        ok = 0;
                        break;
                    }
            aut += ok;
            int i = n - 2;
            while (i >= 0 && p[i] > p[i + 1]) --i;
            if (i < 0) break;
            int j = n - 1;
            while (p[j] < p[i]) --j;
            int t = p[i];
            p[i] = p[j];
            p[j] = t;
            for (int a = i + 1, z = n - 1; a < z; ++a, --z) {
                t = p[a];
                p[a] = p[z];
                p[z] = t;
            }
        }
    }
    i128 total = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : omp_get_max_threads())
    {
        bf_t b = proto;
        b.count = 0;
#pragma omp for schedule(dynamic, 8)
        for (int v = 0; v < V; ++v) {
            b.map[b.order[0]] = v;
            bf_rec(&b, 1);
        }
#pragma omp critical
        total += b.count;
    }
    unsigned __int128 q = (unsigned __int128)total / (unsigned __int128)aut;
    out[0] = (uint64_t)q;
    out[1] = (uint64_t)(q >> 64);
    return 0;
}
