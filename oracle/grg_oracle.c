/*
 * grg_oracle.c -- CPU oracle for the Graspan-G CFL-reachability closure.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: it is loaded by the
 * tests, by the smoke check and by the CPU-baseline leg of the benchmark, and
 * never by the product path (the CUDA library has no reference to it).
 *
 * Parity status: UNPINNED. The reference ships no tests, no golden vectors and
 * no CPU implementation of the closure (its only closure code is GPU code in
 * src/kernel.cu, and its host needs boost, which is absent), so this
 * restatement is checked against an independent pure-Python worklist fixpoint
 * and against hand-derived closures, not against reference output.
 *
 * What it restates (file:line in the reference project):
 *   - grammar file format and label numbering: src/main.cpp:60-97
 *     (lines starting with '#' skipped, first data line = numRules, each rule
 *     "LHS[\tRHS1[\tRHS2]]", labels numbered 1,2,... in order of first
 *     appearance, missing RHS = 0);
 *   - graph file format: src/main.cpp:106-139 and 177-221 (first data line
 *     "numEdges\tnumVars", then numEdges lines "src\tdst\tlabel");
 *   - rule classes: epsilon rules[1]==0 (compute00, src/kernel.cu:445-464),
 *     unary rules[2]==0 (compute10, src/kernel.cu:422-442), binary
 *     (compute11, src/kernel.cu:403-419);
 *   - the 192-id element unit used for all work accounting: 6 bitmap words
 *     per element (src/kernel.h:32-44);
 *   - filter_flag semantics: filter 1 skips every unary rule
 *     (src/kernel.cu:490-494, 698-702, 765-769) and every old-left join
 *     O_B o Delta_C (src/kernel.cu:499-503, 556-562, 592-598, 644-649,
 *     711-716); epsilon rules still run (src/kernel.cu:484-488);
 *   - the final count: the number of distinct (src,dst,label) edges over all
 *     labels, i.e. the popcount of every old-region row (src/main.cpp:909-917,
 *     src/kernel.cu:782-839).
 *
 * Algorithm: round-synchronous semi-naive evaluation. O holds every known
 * edge (including the last round's delta D). Round t computes, per output row
 * (A,i) (owner computes, so rounds are deterministic):
 *     cand = U_{A::=B C} U_{k in D_B[i]} O_C[k]                (delta-left)
 *          U_{A::=B C, C derivable, filter 0} U_{k in O_B[i], D_C[k]!=0} D_C[k]
 *          U_{A::=B, filter 0} D_B[i]
 *     N_A[i] = cand \ O_A[i];  then O |= N, D = N.
 * With filter 0 the fixpoint is the least fixpoint of the grammar. With
 * filter 1 it equals the reference's result exactly when no binary rule's
 * second symbol is derivable (it is then schedule-independent); the oracle
 * refuses other grammars with ORC_E_FILTER.
 */
#define _GNU_SOURCE
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>

#define ORC_OK 0
#define ORC_E_ARG -1
#define ORC_E_FILTER -2
#define ORC_E_NOMEM -3
#define ORC_E_IO -4
#define ORC_E_LABEL -5
#define ORC_E_RANGE -6

#define EW 6            /* bitmap words per element (src/kernel.h:32-33) */
#define EIDS 192        /* ids per element */
#define MAX_RULES 64
#define MAX_LABELS 126
#define NAME_LEN 64
#define NSTAT 8

typedef struct { uint32_t bits[EW]; uint32_t base; uint32_t pad; } oelem;
typedef struct { oelem *e; uint32_t n, cap; } orow;

/* ------------------------------------------------------------------ parsing */

static int read_line(FILE *f, char *buf, size_t cap)
{
    if (!fgets(buf, (int)cap, f)) { buf[0] = 0; return 0; }
    size_t n = strlen(buf);
    while (n && (buf[n - 1] == '\n' || buf[n - 1] == '\r')) buf[--n] = 0;
    return 1;
}

/* skipComments (src/main.cpp:60-67): return the first line not starting with '#'. */
static int next_data_line(FILE *f, char *buf, size_t cap)
{
    for (;;) {
        int ok = read_line(f, buf, cap);
        if (!ok) return 0;
        if (buf[0] != '#') return 1;
    }
}

static int label_lookup(const char *names, int n, const char *s)
{
    for (int i = 0; i < n; i++)
        if (strncmp(names + (size_t)i * NAME_LEN, s, NAME_LEN) == 0) return i + 1;
    return 0;
}

/* readAndTransferRules (src/main.cpp:69-97). names: label l at names[(l-1)*NAME_LEN]. */
int oracle_parse_grammar(const char *path, int *num_rules, int *rules, int *num_labels, char *names)
{
    FILE *f = fopen(path, "r");
    if (!f) return ORC_E_IO;
    char line[4096];
    if (!next_data_line(f, line, sizeof line)) { fclose(f); return ORC_E_IO; }
    int nr = atoi(line);
    if (nr < 0 || nr > MAX_RULES) { fclose(f); return ORC_E_RANGE; }
    int nl = 0;
    memset(rules, 0, sizeof(int) * 3 * MAX_RULES);
    memset(names, 0, (size_t)MAX_LABELS * NAME_LEN);
    for (int r = 0; r < nr; r++) {
        if (!next_data_line(f, line, sizeof line)) { fclose(f); return ORC_E_IO; }
        int j = 0;
        char *p = line;
        for (;;) {
            char *tab = strchr(p, '\t');
            if (tab) *tab = 0;
            if (j < 3 && (*p || tab)) {
                int id = label_lookup(names, nl, p);
                if (!id) {
                    if (nl >= MAX_LABELS || strlen(p) >= NAME_LEN) { fclose(f); return ORC_E_RANGE; }
                    strcpy(names + (size_t)nl * NAME_LEN, p);
                    id = ++nl;
                }
                rules[r * 3 + j] = id;
                j++;
            }
            if (!tab) break;
            p = tab + 1;
        }
        if (rules[r * 3] == 0) { fclose(f); return ORC_E_ARG; }
    }
    fclose(f);
    *num_rules = nr;
    *num_labels = nl;
    return ORC_OK;
}

/* getGraphInfo header (src/main.cpp:106-115). */
int oracle_parse_graph_header(const char *path, uint64_t *num_edges, uint32_t *num_vars)
{
    FILE *f = fopen(path, "r");
    if (!f) return ORC_E_IO;
    char line[4096];
    if (!next_data_line(f, line, sizeof line)) { fclose(f); return ORC_E_IO; }
    char *tab = strchr(line, '\t');
    *num_edges = strtoull(line, NULL, 10);
    *num_vars = tab ? (uint32_t)strtoul(tab + 1, NULL, 10) : 0;
    fclose(f);
    return ORC_OK;
}

/* readEdges (src/main.cpp:177-221), without the sorted-by-src requirement. */
int oracle_parse_graph(const char *path, int num_labels, const char *names, uint64_t num_edges,
                       uint32_t num_vars, uint32_t *src, uint32_t *dst, uint8_t *label)
{
    FILE *f = fopen(path, "r");
    if (!f) return ORC_E_IO;
    char line[4096];
    if (!next_data_line(f, line, sizeof line)) { fclose(f); return ORC_E_IO; }
    for (uint64_t e = 0; e < num_edges; e++) {
        if (!next_data_line(f, line, sizeof line)) { fclose(f); return ORC_E_IO; }
        char *t1 = strchr(line, '\t');
        if (!t1) { fclose(f); return ORC_E_IO; }
        char *t2 = strchr(t1 + 1, '\t');
        if (!t2) { fclose(f); return ORC_E_IO; }
        *t2 = 0;
        char *lab = t2 + 1;
        char *t3 = strchr(lab, '\t');
        if (t3) *t3 = 0;
        unsigned long s = strtoul(line, NULL, 10), d = strtoul(t1 + 1, NULL, 10);
        if (s >= num_vars || d >= num_vars) { fclose(f); return ORC_E_RANGE; }
        int id = label_lookup(names, num_labels, lab);
        if (!id) { fclose(f); return ORC_E_LABEL; }
        src[e] = (uint32_t)s;
        dst[e] = (uint32_t)d;
        label[e] = (uint8_t)id;
    }
    fclose(f);
    return ORC_OK;
}

/* ------------------------------------------------------------ thread pool */

typedef void (*range_fn)(void *ctx, int tid, uint64_t lo, uint64_t hi);
typedef struct { range_fn fn; void *ctx; uint64_t n, grain; atomic_ullong next; int tid; } pf_job;
typedef struct { pf_job *job; int tid; } pf_arg;

static void *pf_worker(void *a)
{
    pf_arg *pa = (pf_arg *)a;
    pf_job *j = pa->job;
    for (;;) {
        uint64_t lo = atomic_fetch_add(&j->next, j->grain);
        if (lo >= j->n) break;
        uint64_t hi = lo + j->grain < j->n ? lo + j->grain : j->n;
        j->fn(j->ctx, pa->tid, lo, hi);
    }
    return NULL;
}

static void parallel_for(int nthreads, uint64_t n, uint64_t grain, range_fn fn, void *ctx)
{
    pf_job job;
    job.fn = fn; job.ctx = ctx; job.n = n; job.grain = grain ? grain : 1;
    atomic_init(&job.next, 0);
    if (nthreads <= 1) {
        pf_arg a = { &job, 0 };
        pf_worker(&a);
        return;
    }
    pthread_t th[256];
    pf_arg args[256];
    if (nthreads > 256) nthreads = 256;
    for (int t = 0; t < nthreads; t++) {
        args[t].job = &job; args[t].tid = t;
        pthread_create(&th[t], NULL, pf_worker, &args[t]);
    }
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------- closure */

typedef struct {
    uint32_t V;
    int L, R, filter, nthreads;
    int rules[3 * MAX_RULES];
    uint8_t derivable[MAX_LABELS + 1];
    uint8_t old_left[MAX_RULES];
    const uint8_t *mask;
    orow *O, *D, *N;           /* [(label-1)*V + row] */
    uint32_t nbases;           /* number of element bases: ceil(V/192) */
    /* per-thread scratch */
    oelem **acc;               /* dense accumulator per thread, nbases entries */
    uint32_t **touched;        /* touched base list per thread */
    uint64_t (*tstat)[NSTAT];  /* per-thread stats of the current round */
    int err;
    /* results */
    uint32_t rounds;
    uint64_t *round_stats;     /* rounds * NSTAT */
    uint64_t label_count[MAX_LABELS + 1];
    uint64_t total, hash;
} oracle_result;

static inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/* Order-independent edge-set hash shared with the CUDA library's self-check. */
static inline uint64_t edge_hash(uint32_t l, uint32_t s, uint32_t d)
{
    return splitmix64(splitmix64(((uint64_t)s << 32) | d) ^ ((uint64_t)l * 0x9E3779B97F4A7C15ull));
}

static inline orow *rowp(orow *base, const oracle_result *r, int label, uint32_t i)
{
    return &base[(size_t)(label - 1) * r->V + i];
}

static int row_reserve(orow *w, uint32_t n)
{
    if (w->cap >= n) return 0;
    uint32_t c = w->cap ? w->cap : 4;
    while (c < n) c *= 2;
    oelem *e = (oelem *)realloc(w->e, sizeof(oelem) * c);
    if (!e) return -1;
    w->e = e; w->cap = c;
    return 0;
}

static inline int cmp_u32(const void *a, const void *b)
{
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return x < y ? -1 : x > y;
}

static inline uint32_t popc6(const uint32_t *b)
{
    uint32_t c = 0;
    for (int w = 0; w < EW; w++) c += (uint32_t)__builtin_popcount(b[w]);
    return c;
}

static inline void acc_or(oracle_result *r, int tid, const oelem *x, uint32_t *nt)
{
    oelem *a = &r->acc[tid][x->base];
    int empty = 1;
    for (int w = 0; w < EW; w++) empty &= (a->bits[w] == 0);
    if (empty) r->touched[tid][(*nt)++] = x->base;
    for (int w = 0; w < EW; w++) a->bits[w] |= x->bits[w];
}

/* Phase 1 of a round: compute N for all output rows with index in [lo,hi). */
static void round_phase1(void *ctx, int tid, uint64_t lo, uint64_t hi)
{
    oracle_result *r = (oracle_result *)ctx;
    uint64_t *st = r->tstat[tid];
    for (uint64_t ii = lo; ii < hi; ii++) {
        uint32_t i = (uint32_t)ii;
        if (r->mask && !r->mask[i]) continue;
        for (int A = 1; A <= r->L; A++) {
            uint32_t nt = 0;
            for (int q = 0; q < r->R; q++) {
                const int *ru = &r->rules[3 * q];
                if (ru[0] != A || ru[1] == 0) continue;
                if (ru[2] == 0) {                       /* unary A ::= B */
                    if (r->filter) continue;
                    orow *db = rowp(r->D, r, ru[1], i);
                    st[6] += db->n;
                    for (uint32_t x = 0; x < db->n; x++) { acc_or(r, tid, &db->e[x], &nt); st[7]++; }
                    continue;
                }
                /* binary A ::= B C, delta-left: D_B[i] o O_C */
                orow *db = rowp(r->D, r, ru[1], i);
                st[2] += db->n;
                for (uint32_t x = 0; x < db->n; x++) {
                    const oelem *el = &db->e[x];
                    for (int w = 0; w < EW; w++) {
                        uint32_t b = el->bits[w];
                        while (b) {
                            int bit = __builtin_ctz(b);
                            b &= b - 1;
                            uint32_t k = el->base * EIDS + (uint32_t)w * 32 + (uint32_t)bit;
                            orow *oc = rowp(r->O, r, ru[2], k);
                            st[3] += oc->n;
                            for (uint32_t y = 0; y < oc->n; y++) { acc_or(r, tid, &oc->e[y], &nt); st[7]++; }
                        }
                    }
                }
                /* old-left: O_B[i] o D_C, only when C is derivable and filter == 0 */
                if (r->old_left[q]) {
                    orow *ob = rowp(r->O, r, ru[1], i);
                    st[4] += ob->n;
                    for (uint32_t x = 0; x < ob->n; x++) {
                        const oelem *el = &ob->e[x];
                        for (int w = 0; w < EW; w++) {
                            uint32_t b = el->bits[w];
                            while (b) {
                                int bit = __builtin_ctz(b);
                                b &= b - 1;
                                uint32_t k = el->base * EIDS + (uint32_t)w * 32 + (uint32_t)bit;
                                orow *dc = rowp(r->D, r, ru[2], k);
                                st[5] += dc->n;
                                for (uint32_t y = 0; y < dc->n; y++) { acc_or(r, tid, &dc->e[y], &nt); st[7]++; }
                            }
                        }
                    }
                }
            }
            if (!nt) continue;
            qsort(r->touched[tid], nt, sizeof(uint32_t), cmp_u32);
            orow *oa = rowp(r->O, r, A, i);
            orow *na = rowp(r->N, r, A, i);
            na->n = 0;
            uint32_t y = 0;
            for (uint32_t t = 0; t < nt; t++) {
                uint32_t base = r->touched[tid][t];
                oelem *a = &r->acc[tid][base];
                while (y < oa->n && oa->e[y].base < base) y++;
                oelem nw; memset(&nw, 0, sizeof nw);
                nw.base = base;
                int any = 0;
                for (int w = 0; w < EW; w++) {
                    uint32_t old = (y < oa->n && oa->e[y].base == base) ? oa->e[y].bits[w] : 0;
                    nw.bits[w] = a->bits[w] & ~old;
                    any |= nw.bits[w] != 0;
                    a->bits[w] = 0;
                }
                if (any) {
                    if (row_reserve(na, na->n + 1)) { r->err = ORC_E_NOMEM; return; }
                    na->e[na->n++] = nw;
                    st[0] += popc6(nw.bits);
                    st[1]++;
                }
            }
        }
    }
}

/* Phase 2: O |= N, D = N. */
static void round_phase2(void *ctx, int tid, uint64_t lo, uint64_t hi)
{
    oracle_result *r = (oracle_result *)ctx;
    (void)tid;
    for (uint64_t ii = lo; ii < hi; ii++) {
        uint32_t i = (uint32_t)ii;
        if (r->mask && !r->mask[i]) continue;
        for (int A = 1; A <= r->L; A++) {
            orow *o = rowp(r->O, r, A, i), *d = rowp(r->D, r, A, i), *n = rowp(r->N, r, A, i);
            d->n = 0;
            if (n->n) {
                orow m = { NULL, 0, 0 };
                if (row_reserve(&m, o->n + n->n)) { r->err = ORC_E_NOMEM; return; }
                uint32_t a = 0, b = 0;
                while (a < o->n || b < n->n) {
                    if (b >= n->n || (a < o->n && o->e[a].base < n->e[b].base)) m.e[m.n++] = o->e[a++];
                    else if (a >= o->n || n->e[b].base < o->e[a].base) m.e[m.n++] = n->e[b++];
                    else {
                        oelem x = o->e[a++];
                        for (int w = 0; w < EW; w++) x.bits[w] |= n->e[b].bits[w];
                        b++;
                        m.e[m.n++] = x;
                    }
                }
                free(o->e);
                *o = m;
            }
            /* swap D and N storage */
            orow t = *d; *d = *n; *n = t;
            n->n = 0;
        }
    }
}

static void free_rows(orow *rows, size_t n)
{
    if (!rows) return;
    for (size_t i = 0; i < n; i++) free(rows[i].e);
    free(rows);
}

void oracle_free(oracle_result *r)
{
    if (!r) return;
    size_t nr = (size_t)r->L * r->V;
    free_rows(r->O, nr);
    free_rows(r->D, nr);
    free_rows(r->N, nr);
    if (r->acc) for (int t = 0; t < r->nthreads; t++) free(r->acc[t]);
    if (r->touched) for (int t = 0; t < r->nthreads; t++) free(r->touched[t]);
    free(r->acc);
    free(r->touched);
    free(r->tstat);
    free(r->round_stats);
    free(r);
}

/* Insert one id into a row kept sorted by base (used only while loading). */
static int row_insert_id(orow *w, uint32_t id)
{
    uint32_t base = id / EIDS, off = id % EIDS;
    uint32_t lo = 0, hi = w->n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (w->e[mid].base < base) lo = mid + 1; else hi = mid;
    }
    if (lo < w->n && w->e[lo].base == base) {
        w->e[lo].bits[off / 32] |= 1u << (off % 32);
        return 0;
    }
    if (row_reserve(w, w->n + 1)) return -1;
    memmove(&w->e[lo + 1], &w->e[lo], sizeof(oelem) * (w->n - lo));
    memset(&w->e[lo], 0, sizeof(oelem));
    w->e[lo].base = base;
    w->e[lo].bits[off / 32] = 1u << (off % 32);
    w->n++;
    return 0;
}

typedef struct { oracle_result *r; const uint64_t *rowstart; const uint32_t *sorted_dst; } load_ctx;

static void load_rows(void *ctx, int tid, uint64_t lo, uint64_t hi)
{
    load_ctx *c = (load_ctx *)ctx;
    (void)tid;
    for (uint64_t q = lo; q < hi; q++) {
        orow *w = &c->r->O[q];
        for (uint64_t e = c->rowstart[q]; e < c->rowstart[q + 1]; e++)
            if (row_insert_id(w, c->sorted_dst[e])) { c->r->err = ORC_E_NOMEM; return; }
    }
}

static void copy_o_to_d(void *ctx, int tid, uint64_t lo, uint64_t hi)
{
    oracle_result *r = (oracle_result *)ctx;
    (void)tid;
    for (uint64_t q = lo; q < hi; q++) {
        orow *o = &r->O[q], *d = &r->D[q];
        if (!o->n) continue;
        if (row_reserve(d, o->n)) { r->err = ORC_E_NOMEM; return; }
        memcpy(d->e, o->e, sizeof(oelem) * o->n);
        d->n = o->n;
    }
}

/*
 * Compute the closure. rules: 3*num_rules label ids (1-based, 0 = absent),
 * as numbered by oracle_parse_grammar. row_mask (nullable): when given, only
 * source rows with mask[i] != 0 are closed and counted; this is only allowed
 * when no rule reads a derivable relation on its right-hand side (rows are
 * then independent), else ORC_E_ARG.
 */
oracle_result *oracle_closure(uint32_t num_vars, int num_labels, int num_rules, const int *rules, int filter,
                              uint64_t num_edges, const uint32_t *src, const uint32_t *dst, const uint8_t *label,
                              const uint8_t *row_mask, int nthreads, int *status)
{
    *status = ORC_OK;
    if (num_labels < 1 || num_labels > MAX_LABELS || num_rules < 0 || num_rules > MAX_RULES || filter < 0 || filter > 1) {
        *status = ORC_E_ARG; return NULL;
    }
    oracle_result *r = (oracle_result *)calloc(1, sizeof(oracle_result));
    if (!r) { *status = ORC_E_NOMEM; return NULL; }
    r->V = num_vars; r->L = num_labels; r->R = num_rules; r->filter = filter;
    r->nthreads = nthreads < 1 ? 1 : nthreads;
    r->mask = row_mask;
    memcpy(r->rules, rules, sizeof(int) * 3 * (size_t)num_rules);
    for (int q = 0; q < num_rules; q++) {
        const int *ru = &r->rules[3 * q];
        if (ru[0] < 1 || ru[0] > num_labels || ru[1] < 0 || ru[1] > num_labels || ru[2] < 0 || ru[2] > num_labels ||
            (ru[1] == 0 && ru[2] != 0)) { *status = ORC_E_ARG; oracle_free(r); return NULL; }
        int is_unary = ru[1] != 0 && ru[2] == 0;
        if (!(filter && is_unary)) r->derivable[ru[0]] = 1;
    }
    int rhs2_derivable = 0;
    for (int q = 0; q < num_rules; q++) {
        const int *ru = &r->rules[3 * q];
        if (ru[1] && ru[2] && r->derivable[ru[2]]) {
            rhs2_derivable = 1;
            r->old_left[q] = filter == 0;
        }
    }
    if (filter && rhs2_derivable) { *status = ORC_E_FILTER; oracle_free(r); return NULL; }
    if (row_mask && rhs2_derivable) { *status = ORC_E_ARG; oracle_free(r); return NULL; }
    for (uint64_t e = 0; e < num_edges; e++)
        if (src[e] >= num_vars || dst[e] >= num_vars || label[e] < 1 || label[e] > num_labels) {
            *status = ORC_E_RANGE; oracle_free(r); return NULL;
        }
    size_t nr = (size_t)num_labels * num_vars;
    r->O = (orow *)calloc(nr ? nr : 1, sizeof(orow));
    r->D = (orow *)calloc(nr ? nr : 1, sizeof(orow));
    r->N = (orow *)calloc(nr ? nr : 1, sizeof(orow));
    r->nbases = (num_vars + EIDS - 1) / EIDS;
    r->acc = (oelem **)calloc((size_t)r->nthreads, sizeof(oelem *));
    r->touched = (uint32_t **)calloc((size_t)r->nthreads, sizeof(uint32_t *));
    r->tstat = calloc((size_t)r->nthreads, sizeof(uint64_t) * NSTAT);
    if (!r->O || !r->D || !r->N || !r->acc || !r->touched || !r->tstat) { *status = ORC_E_NOMEM; oracle_free(r); return NULL; }
    for (int t = 0; t < r->nthreads; t++) {
        r->acc[t] = (oelem *)calloc(r->nbases + 1, sizeof(oelem));
        r->touched[t] = (uint32_t *)malloc(sizeof(uint32_t) * (r->nbases + 1));
        if (!r->acc[t] || !r->touched[t]) { *status = ORC_E_NOMEM; oracle_free(r); return NULL; }
    }

    /* Load: bucket input edges (+ epsilon self-loops) by (label,row). */
    int neps = 0;
    for (int q = 0; q < num_rules; q++) if (r->rules[3 * q + 1] == 0) neps++;
    uint64_t total_in = num_edges + (uint64_t)neps * num_vars;
    uint64_t *rowstart = (uint64_t *)calloc(nr + 1, sizeof(uint64_t));
    uint32_t *sdst = (uint32_t *)malloc(sizeof(uint32_t) * (total_in ? total_in : 1));
    if (!rowstart || !sdst) { free(rowstart); free(sdst); *status = ORC_E_NOMEM; oracle_free(r); return NULL; }
    for (uint64_t e = 0; e < num_edges; e++) rowstart[(size_t)(label[e] - 1) * num_vars + src[e] + 1]++;
    for (int q = 0; q < num_rules; q++)
        if (r->rules[3 * q + 1] == 0)
            for (uint32_t v = 0; v < num_vars; v++) rowstart[(size_t)(r->rules[3 * q] - 1) * num_vars + v + 1]++;
    for (size_t q = 0; q < nr; q++) rowstart[q + 1] += rowstart[q];
    uint64_t *fill = (uint64_t *)malloc(sizeof(uint64_t) * (nr ? nr : 1));
    if (!fill) { free(rowstart); free(sdst); *status = ORC_E_NOMEM; oracle_free(r); return NULL; }
    memcpy(fill, rowstart, sizeof(uint64_t) * nr);
    for (uint64_t e = 0; e < num_edges; e++) sdst[fill[(size_t)(label[e] - 1) * num_vars + src[e]]++] = dst[e];
    for (int q = 0; q < num_rules; q++)
        if (r->rules[3 * q + 1] == 0)
            for (uint32_t v = 0; v < num_vars; v++) sdst[fill[(size_t)(r->rules[3 * q] - 1) * num_vars + v]++] = v;
    free(fill);
    load_ctx lc = { r, rowstart, sdst };
    parallel_for(r->nthreads, nr, 4096, load_rows, &lc);
    free(rowstart);
    free(sdst);
    if (r->err) { *status = r->err; oracle_free(r); return NULL; }
    parallel_for(r->nthreads, nr, 4096, copy_o_to_d, r);
    if (r->err) { *status = r->err; oracle_free(r); return NULL; }

    /* Rounds. */
    uint32_t cap_rounds = 64;
    r->round_stats = (uint64_t *)calloc(cap_rounds * NSTAT, sizeof(uint64_t));
    for (;;) {
        memset(r->tstat, 0, sizeof(uint64_t) * NSTAT * (size_t)r->nthreads);
        parallel_for(r->nthreads, num_vars, 256, round_phase1, r);
        if (r->err) { *status = r->err; oracle_free(r); return NULL; }
        uint64_t s[NSTAT] = { 0 };
        for (int t = 0; t < r->nthreads; t++)
            for (int k = 0; k < NSTAT; k++) s[k] += r->tstat[t][k];
        parallel_for(r->nthreads, num_vars, 1024, round_phase2, r);
        if (r->err) { *status = r->err; oracle_free(r); return NULL; }
        if (r->rounds == cap_rounds) {
            cap_rounds *= 2;
            uint64_t *ns = (uint64_t *)realloc(r->round_stats, sizeof(uint64_t) * NSTAT * cap_rounds);
            if (!ns) { *status = ORC_E_NOMEM; oracle_free(r); return NULL; }
            r->round_stats = ns;
        }
        memcpy(&r->round_stats[(size_t)r->rounds * NSTAT], s, sizeof s);
        r->rounds++;
        if (s[1] == 0) break;
    }

    /* Counts and set hash over the (masked) rows. */
    for (int A = 1; A <= r->L; A++)
        for (uint32_t i = 0; i < num_vars; i++) {
            if (r->mask && !r->mask[i]) continue;
            orow *o = rowp(r->O, r, A, i);
            for (uint32_t x = 0; x < o->n; x++) {
                const oelem *el = &o->e[x];
                r->label_count[A] += popc6(el->bits);
                for (int w = 0; w < EW; w++) {
                    uint32_t b = el->bits[w];
                    while (b) {
                        int bit = __builtin_ctz(b);
                        b &= b - 1;
                        r->hash += edge_hash((uint32_t)A, i, el->base * EIDS + (uint32_t)w * 32 + (uint32_t)bit);
                    }
                }
            }
        }
    for (int A = 1; A <= r->L; A++) r->total += r->label_count[A];
    return r;
}

uint64_t oracle_total(const oracle_result *r) { return r->total; }
uint64_t oracle_set_hash(const oracle_result *r) { return r->hash; }
uint32_t oracle_num_rounds(const oracle_result *r) { return r->rounds; }

void oracle_label_counts(const oracle_result *r, uint64_t *out)
{
    for (int A = 1; A <= r->L; A++) out[A - 1] = r->label_count[A];
}

void oracle_round_stats(const oracle_result *r, uint64_t *out)
{
    memcpy(out, r->round_stats, sizeof(uint64_t) * NSTAT * r->rounds);
}

/*
 * Per-vertex degree like getDegree's old-region columns (src/kernel.cu:782-839):
 * edges[v] = popcount over all labels of row v, elems[v] = number of 192-id
 * elements over all labels of row v.
 */
void oracle_degree(const oracle_result *r, uint32_t *edges, uint32_t *elems)
{
    for (uint32_t i = 0; i < r->V; i++) {
        uint32_t ne = 0, nel = 0;
        for (int A = 1; A <= r->L; A++) {
            const orow *o = &r->O[(size_t)(A - 1) * r->V + i];
            nel += o->n;
            for (uint32_t x = 0; x < o->n; x++) ne += popc6(o->e[x].bits);
        }
        edges[i] = ne;
        elems[i] = nel;
    }
}

/* Export edges sorted by (label, src, dst); returns the number of edges (writes at most cap). */
uint64_t oracle_export(const oracle_result *r, uint32_t *src, uint32_t *dst, uint8_t *label, uint64_t cap)
{
    uint64_t n = 0;
    for (int A = 1; A <= r->L; A++)
        for (uint32_t i = 0; i < r->V; i++) {
            if (r->mask && !r->mask[i]) continue;
            const orow *o = &r->O[(size_t)(A - 1) * r->V + i];
            for (uint32_t x = 0; x < o->n; x++) {
                const oelem *el = &o->e[x];
                for (int w = 0; w < EW; w++) {
                    uint32_t b = el->bits[w];
                    while (b) {
                        int bit = __builtin_ctz(b);
                        b &= b - 1;
                        if (n < cap) {
                            src[n] = i;
                            dst[n] = el->base * EIDS + (uint32_t)w * 32 + (uint32_t)bit;
                            label[n] = (uint8_t)A;
                        }
                        n++;
                    }
                }
            }
        }
    return n;
}

uint64_t oracle_edge_hash(uint32_t l, uint32_t s, uint32_t d) { return edge_hash(l, s, d); }

/*
 * Closure edges of source rows [v_begin, v_end) in the reference's compressed
 * spill format: elements2Edges (src/main.cpp:510-539) as storeElements_c
 * (src/main.cpp:541-596) lays it out. For each source vertex in order, for
 * each label 1..L, the row's elements in base order and each element's ids
 * ascending: 5 bytes per edge, the destination as a little-endian uint32, then
 * the label id. degree[v - v_begin] = the vertex's edge count, the row lengths
 * readElements_c (src/main.cpp:364-372) reads the stream back with. Returns the
 * number of edges; writes at most cap of them (degree always in full).
 */
uint64_t oracle_export_csr5(const oracle_result *r, uint32_t v_begin, uint32_t v_end, uint8_t *out,
                            uint32_t *degree, uint64_t cap)
{
    uint64_t n = 0;
    for (uint32_t i = v_begin; i < v_end && i < r->V; i++) {
        uint32_t deg = 0;
        for (int A = 1; A <= r->L; A++) {
            const orow *o = &r->O[(size_t)(A - 1) * r->V + i];
            for (uint32_t x = 0; x < o->n; x++) {
                const oelem *el = &o->e[x];
                for (int w = 0; w < EW; w++) {
                    uint32_t b = el->bits[w];
                    while (b) {
                        const int bit = __builtin_ctz(b);
                        b &= b - 1;
                        if (n < cap && out) {
                            const uint32_t dst = el->base * EIDS + (uint32_t)w * 32 + (uint32_t)bit;
                            uint8_t *q = out + n * 5;
                            q[0] = (uint8_t)dst;
                            q[1] = (uint8_t)(dst >> 8);
                            q[2] = (uint8_t)(dst >> 16);
                            q[3] = (uint8_t)(dst >> 24);
                            q[4] = (uint8_t)A;
                        }
                        n++;
                        deg++;
                    }
                }
            }
        }
        if (degree) degree[i - v_begin] = deg;
    }
    return n;
}

