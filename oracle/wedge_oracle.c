/*
 * ORACLE -- test infrastructure, not product code.  See wedge_oracle.h.
 *
 * Portable-C restatement of the reference's pull-only edge-pull engine.  It
 * keeps the reference's data layout (4-lane "edge vectors" of 64-bit words,
 * vertex index, CSRI, Wedge frontier of one bit per 4 vectors, traditional
 * bitmaps, per-thread reduce buffer, per-work-unit merge buffers) and its SPMD
 * control flow (32 dynamically scheduled work units per thread, barriers
 * between phases), with every AVX2 lane operation written as a scalar loop.
 *
 * Deviations, all deliberate:
 *  - A dense CC/SSSP work unit that holds no vector is skipped; the reference
 *    indexes graph_vertex_props[UINT64_MAX] there (phase_edge_pull_cc.c:139-142,
 *    phase_edge_pull_sssp.c:146-149) when a graph has < 32*threads vectors.
 *  - PageRank's damping is a parameter (the reference hard-codes 0.875,
 *    include/constants.h:39).
 *  - SSSP has an FP64-weight variant (double min-plus); the reference has
 *    only uint64 weights (phase_edge_pull_sssp.c:93,137).
 * Everything else follows the cited reference lines.
 */
#define _GNU_SOURCE
#include "wedge_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdbool.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

#define VALID_BIT 0x8000000000000000ull
#define SRC_MASK 0x0000ffffffffffffull
#define LOG2_PRECISION 2ull /* include/configuration.h:19-24 */

/* ======================================================================== */
/* generators                                                               */
/* ======================================================================== */

/* splitmix64 finaliser (Steele, Lea, Flood 2014) */
uint64_t orc_mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* counter-based draw: word `word` (< 16) of item `item` under `seed` */
uint64_t orc_draw(uint64_t seed, uint64_t item, uint64_t word)
{
    return orc_mix64(orc_mix64(seed) + ((item << 4) | (word & 15ull)));
}

void orc_rmat_thresholds(double a, double b, double c, uint64_t out[3])
{
    out[0] = (uint64_t)(a * 4294967296.0);
    out[1] = (uint64_t)((a + b) * 4294967296.0);
    out[2] = (uint64_t)((a + b + c) * 4294967296.0);
}

typedef struct {
    uint32_t scale;
    uint64_t t[3], seed, first, count;
    uint32_t *src, *dst;
    int threads, id;
} rmat_job_t;

static inline uint64_t mix64_inline(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void* rmat_worker(void* p)
{
    rmat_job_t* j = (rmat_job_t*)p;
    const uint64_t hseed = mix64_inline(j->seed); /* orc_draw's first mix, hoisted */
    const uint64_t per = j->count / j->threads, extra = j->count % j->threads;
    const uint64_t lo = per * j->id + ((uint64_t)j->id < extra ? j->id : extra);
    const uint64_t hi = lo + per + ((uint64_t)j->id < extra ? 1 : 0);
    for (uint64_t k = lo; k < hi; ++k) {
        const uint64_t e = j->first + k;
        uint32_t s = 0, d = 0;
        uint64_t h = 0;
        for (uint32_t l = 0; l < j->scale; ++l) {
            if ((l & 1u) == 0)
                h = mix64_inline(hseed + ((e << 4) | (l >> 1))); /* == orc_draw(seed, e, l/2) */
            const uint64_t u = (l & 1u) ? (h >> 32) : (h & 0xffffffffull);
            const uint32_t bit = 1u << (j->scale - 1 - l);
            if (u < j->t[0]) {
            } else if (u < j->t[1]) {
                d |= bit;
            } else if (u < j->t[2]) {
                s |= bit;
            } else {
                s |= bit;
                d |= bit;
            }
        }
        j->src[k] = s;
        j->dst[k] = d;
    }
    return NULL;
}

/*
 * R-MAT edge list: edge e chooses one quadrant per bit level, most significant
 * bit first, from the 32-bit halves of orc_draw(seed, e, level/2).  Quadrants
 * a/b/c/d are (src,dst) bit pairs (0,0)/(0,1)/(1,0)/(1,1).  No noise, no
 * relabelling; duplicates and self-loops are kept.
 */
void orc_rmat(uint32_t scale, double a, double b, double c, uint64_t seed, uint64_t first,
              uint64_t count, uint32_t* src, uint32_t* dst, int threads)
{
    if (threads <= 0)
        threads = orc_online_cores();
    rmat_job_t* jobs = (rmat_job_t*)calloc((size_t)threads, sizeof(rmat_job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int i = 0; i < threads; ++i) {
        jobs[i].scale = scale;
        orc_rmat_thresholds(a, b, c, jobs[i].t);
        jobs[i].seed = seed;
        jobs[i].first = first;
        jobs[i].count = count;
        jobs[i].src = src;
        jobs[i].dst = dst;
        jobs[i].threads = threads;
        jobs[i].id = i;
        pthread_create(&th[i], NULL, rmat_worker, &jobs[i]);
    }
    for (int i = 0; i < threads; ++i)
        pthread_join(th[i], NULL);
    free(jobs);
    free(th);
}

static uint64_t mulhi64(uint64_t a, uint64_t b)
{
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
}

uint64_t orc_grid_edge_count(uint64_t side, double long_range_frac)
{
    const uint64_t base = 4ull * side * (side - 1ull);
    return base + (uint64_t)(long_range_frac * (double)base);
}

/*
 * side x side grid, vertex r*side+c, both directions of every 4-neighbour
 * pair (right then down per vertex, row-major), followed by
 * floor(frac * 4*side*(side-1)) uniform directed long-range pairs drawn with
 * orc_draw(seed, i, 0/1) scaled by a 64x64->128 multiply-high.
 */
void orc_grid(uint64_t side, double long_range_frac, uint64_t seed, uint32_t* src, uint32_t* dst)
{
    const uint64_t V = side * side;
    const uint64_t base = 4ull * side * (side - 1ull);
    const uint64_t lr = (uint64_t)(long_range_frac * (double)base);
    uint64_t k = 0;
    for (uint64_t r = 0; r < side; ++r) {
        for (uint64_t c = 0; c < side; ++c) {
            const uint64_t v = r * side + c;
            if (c + 1 < side) {
                src[k] = (uint32_t)v;
                dst[k++] = (uint32_t)(v + 1);
                src[k] = (uint32_t)(v + 1);
                dst[k++] = (uint32_t)v;
            }
            if (r + 1 < side) {
                src[k] = (uint32_t)v;
                dst[k++] = (uint32_t)(v + side);
                src[k] = (uint32_t)(v + side);
                dst[k++] = (uint32_t)v;
            }
        }
    }
    for (uint64_t i = 0; i < lr; ++i) {
        src[k] = (uint32_t)mulhi64(orc_draw(seed, i, 0), V);
        dst[k++] = (uint32_t)mulhi64(orc_draw(seed, i, 1), V);
    }
}

/* multiplicative hash of (src,dst), high bits kept: w in [1,255] */
uint64_t orc_weight_u64(uint64_t s, uint64_t d)
{
    const uint64_t h = ((s << 32) | d) * 0x9E3779B97F4A7C15ull;
    return 1ull + (((h >> 32) * 255ull) >> 32);
}

/* same hash as a double in [0,1]: h * 2^-64 */
double orc_weight_f64(uint64_t s, uint64_t d)
{
    const uint64_t h = ((s << 32) | d) * 0x9E3779B97F4A7C15ull;
    return (double)h * 0x1p-64;
}

void orc_weights(uint64_t E, const uint32_t* src, const uint32_t* dst, int kind, uint64_t* out)
{
    for (uint64_t e = 0; e < E; ++e) {
        if (kind == ORC_WEIGHTS_F64) {
            const double w = orc_weight_f64(src[e], dst[e]);
            memcpy(&out[e], &w, 8);
        } else {
            out[e] = orc_weight_u64(src[e], dst[e]);
        }
    }
}

/* ---- parallel LSD radix sort of (dst<<32 | src) keys, 11-bit digits ---- */
typedef struct {
    uint64_t *in, *out, n;
    uint64_t* hist; /* threads x 2048 */
    int threads, id, shift;
    pthread_barrier_t* bar;
} sort_job_t;

static void* sort_worker(void* p)
{
    sort_job_t* j = (sort_job_t*)p;
    const uint64_t per = j->n / j->threads, extra = j->n % j->threads;
    const uint64_t lo = per * j->id + ((uint64_t)j->id < extra ? j->id : extra);
    const uint64_t hi = lo + per + ((uint64_t)j->id < extra ? 1 : 0);
    uint64_t* h = &j->hist[(size_t)j->id * 2048];
    memset(h, 0, 2048 * sizeof(uint64_t));
    for (uint64_t i = lo; i < hi; ++i)
        h[(j->in[i] >> j->shift) & 2047ull]++;
    pthread_barrier_wait(j->bar);
    if (j->id == 0) {
        uint64_t run = 0;
        for (int dgt = 0; dgt < 2048; ++dgt) {
            for (int t = 0; t < j->threads; ++t) {
                const uint64_t c = j->hist[(size_t)t * 2048 + dgt];
                j->hist[(size_t)t * 2048 + dgt] = run;
                run += c;
            }
        }
    }
    pthread_barrier_wait(j->bar);
    for (uint64_t i = lo; i < hi; ++i) {
        const uint64_t k = j->in[i];
        j->out[h[(k >> j->shift) & 2047ull]++] = k;
    }
    return NULL;
}

int orc_sort_edges(uint64_t V, uint64_t E, uint32_t* src, uint32_t* dst, int threads)
{
    if (threads <= 0)
        threads = orc_online_cores();
    uint64_t* a = (uint64_t*)malloc(E * 8 + 8);
    uint64_t* b = (uint64_t*)malloc(E * 8 + 8);
    uint64_t* hist = (uint64_t*)malloc((size_t)threads * 2048 * 8);
    if (!a || !b || !hist) {
        free(a);
        free(b);
        free(hist);
        return ORC_ERR_OOM;
    }
    for (uint64_t e = 0; e < E; ++e)
        a[e] = ((uint64_t)dst[e] << 32) | src[e];
    int bits = 1;
    while (bits < 64 && (1ull << bits) < V)
        ++bits;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)threads);
    sort_job_t* jobs = (sort_job_t*)calloc((size_t)threads, sizeof(sort_job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    /* source digits cover bits [0,bits), destination digits [32,32+bits) */
    int shifts[12], ns = 0;
    for (int s = 0; s < bits; s += 11)
        shifts[ns++] = s;
    for (int s = 0; s < bits; s += 11)
        shifts[ns++] = 32 + s;
    for (int pass = 0; pass < ns; ++pass) {
        for (int i = 0; i < threads; ++i) {
            jobs[i] = (sort_job_t){a, b, E, hist, threads, i, shifts[pass], &bar};
            pthread_create(&th[i], NULL, sort_worker, &jobs[i]);
        }
        for (int i = 0; i < threads; ++i)
            pthread_join(th[i], NULL);
        uint64_t* t = a;
        a = b;
        b = t;
    }
    pthread_barrier_destroy(&bar);
    for (uint64_t e = 0; e < E; ++e) {
        dst[e] = (uint32_t)(a[e] >> 32);
        src[e] = (uint32_t)a[e];
    }
    free(jobs);
    free(th);
    free(a);
    free(b);
    free(hist);
    return ORC_OK;
}

void orc_symmetrise(uint64_t E, uint32_t* src, uint32_t* dst)
{
    for (uint64_t e = 0; e < E; ++e) {
        src[E + e] = dst[e];
        dst[E + e] = src[e];
    }
}

int orc_write_file(const char* path, uint64_t V, uint64_t E, const uint32_t* src, const uint32_t* dst,
                   const uint64_t* weights)
{
    FILE* f = fopen(path, "wb");
    if (!f)
        return ORC_ERR_IO;
    const uint64_t hdr[2] = {V, E};
    fwrite(hdr, 8, 2, f);
    uint64_t buf[3 * 4096];
    const uint64_t tup = weights ? 3 : 2;
    uint64_t n = 0;
    for (uint64_t e = 0; e < E; ++e) {
        buf[n++] = src[e];
        buf[n++] = dst[e];
        if (weights)
            buf[n++] = weights[e];
        if (n == tup * 4096) {
            fwrite(buf, 8, n, f);
            n = 0;
        }
    }
    if (n)
        fwrite(buf, 8, n, f);
    const int bad = ferror(f);
    fclose(f);
    return bad ? ORC_ERR_IO : ORC_OK;
}

/* ======================================================================== */
/* engine                                                                   */
/* ======================================================================== */

typedef struct {
    uint64_t initial_vertex_id;
    uint64_t final_vertex_id;
    uint64_t final_partial_value;
    uint64_t pad;
} mergeaccum_t; /* include/graphtypes.h:34-41 */

struct orc_graph {
    uint64_t V, E, nvec, nvec_alloc;
    int weighted;
    uint64_t* vec;        /* graph_edges_gather_list_bufs_numa[0] */
    uint64_t* index;      /* graph_edges_gather_list_index_numa[0] */
    uint64_t* outdeg;     /* graph_vertex_outdegrees */
    uint64_t* props;      /* graph_vertex_props */
    uint64_t* acc;        /* graph_vertex_accumulators */
    uint64_t* csri_index; /* graph_edges_wedge_csri_index_numa[0] */
    uint64_t* csri_edges; /* graph_edges_wedge_csri_edges_numa[0] */
    uint64_t* wedge;      /* graph_wedge_frontier_numa[0] */
    uint64_t wedge_count;
    uint64_t* active;     /* graph_frontier_active_vertices */
    uint64_t* snapshot;   /* graph_frontier_active_vertices_snapshot */
    uint64_t* unconverged;
    uint64_t frontier_count;
    int outdeg_f64; /* execution_initialize_pr turned the out-degree words into doubles */
};

/* per-run shared state (the reference keeps it in globals) */
typedef struct {
    orc_graph_t* g;
    orc_params_t p;
    int app;
    int threads;
    pthread_barrier_t bar;
    uint64_t dyn; /* graph_scheduler_dynamic_counter_numa[0] */
    uint64_t* reduce;
    mergeaccum_t* merge;
    orc_stats_t stats;
    double damping;
} run_t;

static __thread int t_id;

static void barrier(run_t* r) { pthread_barrier_wait(&r->bar); }

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC_RAW, &ts);
    return (double)ts.tv_sec * 1000.0 + (double)ts.tv_nsec / 1e6;
}

int orc_online_cores(void)
{
    long n = sysconf(_SC_NPROCESSORS_ONLN);
    return n > 0 ? (int)n : 1;
}

static inline uint64_t dst_of(const uint64_t* w) /* graphdata.c:49-55 */
{
    return ((w[0] & 0x7fff000000000000ull) >> 48) | ((w[1] & 0x7fff000000000000ull) >> 33) |
           ((w[2] & 0x7fff000000000000ull) >> 18) | ((w[3] & 0x0007000000000000ull) >> 3);
}

static inline void set_bit(uint64_t* bm, uint64_t i)
{
    uint8_t* a = &((uint8_t*)bm)[i >> 3];
    __atomic_fetch_or(a, (uint8_t)(1u << (i & 7)), __ATOMIC_RELAXED);
}

static inline int cond_set_bit(uint64_t* bm, uint64_t i) /* returns previous bit */
{
    uint8_t* a = &((uint8_t*)bm)[i >> 3];
    const uint8_t m = (uint8_t)(1u << (i & 7));
    if (__atomic_load_n(a, __ATOMIC_RELAXED) & m)
        return 1;
    __atomic_fetch_or(a, m, __ATOMIC_RELAXED);
    return 0;
}

static inline void clear_bit(uint64_t* bm, uint64_t i)
{
    uint8_t* a = &((uint8_t*)bm)[i >> 3];
    __atomic_fetch_and(a, (uint8_t)~(1u << (i & 7)), __ATOMIC_RELAXED);
}

static inline int test_bit(const uint64_t* bm, uint64_t i) { return (int)((bm[i >> 6] >> (i & 63)) & 1ull); }

static inline double as_d(uint64_t u)
{
    double d;
    memcpy(&d, &u, 8);
    return d;
}

static inline uint64_t as_u(double d)
{
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
}

/* graphdata.c:212-243: compose one edge vector (and its weight vector) */
static void write_edge_vector(uint64_t dst, const uint64_t* srcs, const uint64_t* wts, uint64_t count,
                              int weighted, uint64_t* out)
{
    const uint64_t pieces[4] = {dst & 0x7fffull, (dst >> 15) & 0x7fffull, (dst >> 30) & 0x7fffull,
                                (dst >> 45) & 0x7ull};
    for (int k = 0; k < 4; ++k)
        out[k] = ((count > (uint64_t)k ? 1ull : 0ull) << 63) | (pieces[k] << 48) | (srcs[k] & SRC_MASK);
    if (weighted)
        for (int k = 0; k < 4; ++k)
            out[4 + k] = count > (uint64_t)k ? wts[k] : 0ull;
}

static void* xalloc(size_t bytes, int fill)
{
    void* p = NULL;
    size_t r = (bytes + 4095) & ~(size_t)4095;
    if (r == 0)
        r = 4096;
    if (posix_memalign(&p, 4096, r) != 0)
        return NULL;
    memset(p, fill, r);
    return p;
}

void orc_free(orc_graph_t* g)
{
    if (!g)
        return;
    free(g->vec);
    free(g->index);
    free(g->outdeg);
    free(g->props);
    free(g->acc);
    free(g->csri_index);
    free(g->csri_edges);
    free(g->wedge);
    free(g->active);
    free(g->snapshot);
    free(g->unconverged);
    free(g);
}

/* ---- a small parallel-for over pthreads (the reference uses Spindle tasks) ---- */
typedef struct {
    void (*fn)(void* ctx, int id, int n);
    void* ctx;
    int id, n;
} pf_job_t;

static void* pf_main(void* p)
{
    pf_job_t* j = (pf_job_t*)p;
    j->fn(j->ctx, j->id, j->n);
    return NULL;
}

static void parallel_run(int n, void (*fn)(void*, int, int), void* ctx)
{
    pf_job_t* jobs = (pf_job_t*)calloc((size_t)n, sizeof(pf_job_t));
    pthread_t* th = (pthread_t*)calloc((size_t)n, sizeof(pthread_t));
    for (int i = 0; i < n; ++i)
        jobs[i] = (pf_job_t){fn, ctx, i, n};
    for (int i = 1; i < n; ++i)
        pthread_create(&th[i], NULL, pf_main, &jobs[i]);
    pf_main(&jobs[0]);
    for (int i = 1; i < n; ++i)
        pthread_join(th[i], NULL);
    free(jobs);
    free(th);
}

static inline void chunk_of(uint64_t total, int id, int n, uint64_t* lo, uint64_t* hi)
{
    const uint64_t per = total / (uint64_t)n, extra = total % (uint64_t)n;
    *lo = per * (uint64_t)id + ((uint64_t)id < extra ? (uint64_t)id : extra);
    *hi = *lo + per + ((uint64_t)id < extra ? 1 : 0);
}

typedef struct {
    orc_graph_t* g;
    const uint32_t* src;
    const uint32_t* dst;
    const uint64_t* w;
    uint64_t* cut;  /* [n+1] edge positions, each at the start of a destination run */
    uint64_t* voff; /* [n+1] vectors before part p (after the prefix) */
    int* err;
} build_ctx_t;

/* validation and vector count of one part (graphdata.c:1017-1035, first pass) */
static void bp_count(void* p, int id, int n)
{
    (void)n;
    build_ctx_t* c = (build_ctx_t*)p;
    const uint64_t V = c->g->V;
    uint64_t nvec = 0, run = 0;
    for (uint64_t e = c->cut[id]; e < c->cut[id + 1]; ++e) {
        if (c->dst[e] >= V || c->src[e] >= V)
            c->err[id] = ORC_ERR_FORMAT;
        if (e > 0 && c->dst[e] != c->dst[e - 1]) {
            if (c->dst[e] < c->dst[e - 1])
                c->err[id] = ORC_ERR_FORMAT; /* input must be grouped by ascending dst */
            if (e != c->cut[id])
                nvec += (run + 3) / 4;
            run = 0;
        }
        ++run;
    }
    if (run)
        nvec += (run + 3) / 4;
    c->voff[id + 1] = nvec;
}

/* second pass: a stash of up to 4 sources per destination run (graphdata.c:247-319) */
static void bp_pack(void* p, int id, int n)
{
    (void)n;
    build_ctx_t* c = (build_ctx_t*)p;
    orc_graph_t* g = c->g;
    const uint64_t words = g->weighted ? 8 : 4;
    uint64_t stash_s[4] = {0}, stash_w[4] = {0}, stash_d = 0, cnt = 0, wi = c->voff[id];
    for (uint64_t e = c->cut[id]; e < c->cut[id + 1]; ++e) {
        if ((cnt != 0 && stash_d != c->dst[e]) || cnt == 4) {
            write_edge_vector(stash_d, stash_s, stash_w, cnt, g->weighted, &g->vec[wi * words]);
            ++wi;
            cnt = 0;
        }
        stash_d = c->dst[e];
        stash_s[cnt] = c->src[e];
        stash_w[cnt] = c->w ? c->w[e] : 0;
        ++cnt;
    }
    if (cnt)
        write_edge_vector(stash_d, stash_s, stash_w, cnt, g->weighted, &g->vec[wi * words]);
}

/* vertex index (graphdata.c:402-427) and out-degrees (graphdata.c:430-490) */
static void bp_index(void* p, int id, int n)
{
    build_ctx_t* c = (build_ctx_t*)p;
    orc_graph_t* g = c->g;
    const uint64_t words = g->weighted ? 8 : 4;
    uint64_t lo, hi;
    chunk_of(g->nvec, id, n, &lo, &hi);
    uint64_t last = lo > 0 ? dst_of(&g->vec[(lo - 1) * words]) : UINT64_MAX;
    for (uint64_t i = lo; i < hi; ++i) {
        const uint64_t d = dst_of(&g->vec[i * words]);
        if (d != last) {
            g->index[d] = i;
            last = d;
        }
        for (int k = 0; k < 4; ++k) {
            const uint64_t x = g->vec[i * words + k];
            if (x & VALID_BIT)
                __atomic_fetch_add(&g->outdeg[x & SRC_MASK], 1ull, __ATOMIC_RELAXED);
        }
    }
}

/* CSRI fill with an atomic cursor per source (graphdata.c:535-569) */
static void bp_csri(void* p, int id, int n)
{
    build_ctx_t* c = (build_ctx_t*)p;
    orc_graph_t* g = c->g;
    const uint64_t words = g->weighted ? 8 : 4;
    uint64_t lo, hi;
    chunk_of(g->nvec, id, n, &lo, &hi);
    for (uint64_t i = lo; i < hi; ++i)
        for (int k = 0; k < 4; ++k) {
            const uint64_t x = g->vec[i * words + k];
            if (x & VALID_BIT) {
                const uint64_t pos = __atomic_fetch_add(&g->csri_index[x & SRC_MASK], 1ull, __ATOMIC_RELAXED);
                g->csri_edges[pos] = i >> LOG2_PRECISION;
            }
        }
}

/*
 * graphdata.c:946-1133 (+ :648-942): pack dst-grouped edges into vectors, pad to
 * a multiple of 4 vectors with invalid vectors of dst V-1, then build the
 * vertex index (:402-427), out-degrees (:430-490), CSRI (:493-585), the Wedge
 * frontier (:804-842) and the traditional bitmaps (:845-892).
 */
static int build_common(orc_graph_t* g, const uint32_t* src, const uint32_t* dst, const uint64_t* w, int threads)
{
    const uint64_t V = g->V, E = g->E;
    int n = threads > 0 ? threads : orc_online_cores();
    if ((uint64_t)n > E / 4096 + 1)
        n = (int)(E / 4096 + 1);
    build_ctx_t c = {g, src, dst, w, NULL, NULL, NULL};
    c.cut = (uint64_t*)calloc((size_t)n + 1, 8);
    c.voff = (uint64_t*)calloc((size_t)n + 1, 8);
    c.err = (int*)calloc((size_t)n, sizeof(int));
    if (!c.cut || !c.voff || !c.err) {
        free(c.cut);
        free(c.voff);
        free(c.err);
        return ORC_ERR_OOM;
    }
    for (int i = 1; i < n; ++i) {
        uint64_t b = E * (uint64_t)i / (uint64_t)n;
        if (b < c.cut[i - 1])
            b = c.cut[i - 1];
        while (b > 0 && b < E && dst[b] == dst[b - 1])
            ++b;
        c.cut[i] = b;
    }
    c.cut[n] = E;
    parallel_run(n, bp_count, &c);
    int rc = ORC_OK;
    for (int i = 0; i < n; ++i)
        if (c.err[i])
            rc = c.err[i];
    for (int i = 0; i < n; ++i)
        c.voff[i + 1] += c.voff[i];
    const uint64_t nvec = c.voff[n];
    if (rc == ORC_OK) {
        g->nvec = nvec;
        g->nvec_alloc = nvec + (4ull - (nvec & 3ull));
        g->vec = (uint64_t*)xalloc(g->nvec_alloc * (g->weighted ? 8 : 4) * 8, 0);
        if (!g->vec)
            rc = ORC_ERR_OOM;
    }
    if (rc == ORC_OK) {
        const uint64_t words = g->weighted ? 8 : 4;
        const uint64_t zero[4] = {0, 0, 0, 0};
        for (uint64_t i = nvec; i < g->nvec_alloc; ++i)
            write_edge_vector(V - 1, zero, zero, 0, g->weighted, &g->vec[i * words]);
        parallel_run(n, bp_pack, &c);
        const uint64_t Va = V + (8ull - (V & 7ull));
        g->index = (uint64_t*)xalloc(Va * 8, 0xff);
        g->outdeg = (uint64_t*)xalloc(Va * 8, 0);
        g->props = (uint64_t*)xalloc(Va * 8, 0);
        g->acc = (uint64_t*)xalloc(Va * 8, 0);
        /* Wedge frontier: (nvec >> 11) + 1 blocks of 512 bits (graphdata.c:810-819) */
        const uint64_t blocks = (nvec >> (9ull + LOG2_PRECISION)) + 1ull;
        g->wedge_count = blocks * 8ull;
        g->wedge = (uint64_t*)xalloc(g->wedge_count * 8, 0);
        g->csri_index = (uint64_t*)xalloc((V + 1) * 8, 0);
        g->csri_edges = (uint64_t*)xalloc((nvec * 4 + 1) * 8, 0);
        const uint64_t fbytes = ((V >> 9) + ((V & 511ull) ? 1 : 0)) << 6;
        g->frontier_count = fbytes >> 3;
        g->active = (uint64_t*)xalloc(fbytes + 64, 0);
        g->snapshot = (uint64_t*)xalloc(fbytes + 64, 0);
        g->unconverged = (uint64_t*)xalloc(fbytes + 64, 0xff);
        if (!g->index || !g->outdeg || !g->props || !g->acc || !g->wedge || !g->csri_index || !g->csri_edges ||
            !g->active || !g->snapshot || !g->unconverged)
            rc = ORC_ERR_OOM;
    }
    if (rc == ORC_OK) {
        parallel_run(n, bp_index, &c);
        uint64_t pos = 0;
        for (uint64_t v = 0; v < V; ++v) {
            g->csri_index[v] = pos;
            pos += g->outdeg[v];
        }
        g->csri_index[V] = pos;
        parallel_run(n, bp_csri, &c);
        pos = 0;
        for (uint64_t v = 0; v < V; ++v) {
            g->csri_index[v] = pos;
            pos += g->outdeg[v];
        }
        g->csri_index[V] = pos;
    }
    free(c.cut);
    free(c.voff);
    free(c.err);
    return rc;
}

int orc_build(uint64_t V, uint64_t E, const uint32_t* src, const uint32_t* dst, const uint64_t* weights,
              int app, int threads, orc_graph_t** out)
{
    *out = NULL;
    if (V == 0)
        return ORC_ERR_FORMAT;
    orc_graph_t* g = (orc_graph_t*)calloc(1, sizeof(orc_graph_t));
    if (!g)
        return ORC_ERR_OOM;
    g->V = V;
    g->E = E;
    g->weighted = (app == ORC_SSSP); /* application.c:171 */
    uint64_t* w = NULL;
    if (g->weighted && !weights) {
        w = (uint64_t*)malloc(E * 8 + 8);
        if (!w) {
            orc_free(g);
            return ORC_ERR_OOM;
        }
        orc_weights(E, src, dst, ORC_WEIGHTS_U64, w);
    }
    const int rc = build_common(g, src, dst, weights ? weights : w, threads);
    free(w);
    if (rc != ORC_OK) {
        orc_free(g);
        return rc;
    }
    *out = g;
    return ORC_OK;
}

/* graphdata.c:589-642 + :946-979: header, exact size check, then the records */
int orc_load_file(const char* path, int app, int threads, orc_graph_t** out)
{
    *out = NULL;
    FILE* f = fopen(path, "rb");
    if (!f)
        return ORC_ERR_IO;
    uint64_t hdr[2];
    if (fread(hdr, 8, 2, f) != 2) {
        fclose(f);
        return ORC_ERR_FORMAT;
    }
    fseek(f, 0, SEEK_END);
    const long fsize = ftell(f);
    fseek(f, 16, SEEK_SET);
    const uint64_t tup = (app == ORC_SSSP) ? 3 : 2;
    if (hdr[1] > ((uint64_t)1 << 40) || (uint64_t)fsize != 16 + hdr[1] * tup * 8 || hdr[0] > 0xffffffffull) {
        fclose(f);
        return ORC_ERR_FORMAT;
    }
    const uint64_t V = hdr[0], E = hdr[1];
    uint32_t* src = (uint32_t*)malloc(E * 4 + 4);
    uint32_t* dst = (uint32_t*)malloc(E * 4 + 4);
    uint64_t* w = tup == 3 ? (uint64_t*)malloc(E * 8 + 8) : NULL;
    uint64_t* buf = (uint64_t*)malloc(3 * 65536 * 8);
    if (!src || !dst || (tup == 3 && !w) || !buf) {
        free(src);
        free(dst);
        free(w);
        free(buf);
        fclose(f);
        return ORC_ERR_OOM;
    }
    int rc = ORC_OK;
    for (uint64_t e = 0; e < E && rc == ORC_OK;) {
        const uint64_t n = (E - e) < 65536 ? (E - e) : 65536;
        if (fread(buf, 8, n * tup, f) != n * tup) {
            rc = ORC_ERR_IO;
            break;
        }
        for (uint64_t i = 0; i < n; ++i) {
            const uint64_t s = buf[i * tup], d = buf[i * tup + 1];
            if (s >= V || d >= V) {
                rc = ORC_ERR_FORMAT;
                break;
            }
            src[e + i] = (uint32_t)s;
            dst[e + i] = (uint32_t)d;
            if (w)
                w[e + i] = buf[i * tup + 2];
        }
        e += n;
    }
    fclose(f);
    free(buf);
    if (rc == ORC_OK)
        rc = orc_build(V, E, src, dst, w, app, threads, out);
    free(src);
    free(dst);
    free(w);
    return rc;
}

uint64_t orc_num_vertices(const orc_graph_t* g) { return g->V; }
uint64_t orc_num_edges(const orc_graph_t* g) { return g->E; }
uint64_t orc_num_edge_vectors(const orc_graph_t* g) { return g->nvec; }
const uint64_t* orc_props(const orc_graph_t* g) { return g->props; }
const uint64_t* orc_outdegrees(const orc_graph_t* g) { return g->outdeg; }
const uint64_t* orc_edge_vectors(const orc_graph_t* g, uint64_t* words)
{
    *words = g->nvec_alloc * (g->weighted ? 8 : 4);
    return g->vec;
}

/* ---- schedule helpers (phase_edge_pull_bfs.c:120-137) ---- */
typedef struct {
    uint64_t units, per, extra;
} sched_t;

static inline sched_t sched_make(uint64_t work, uint64_t units)
{
    sched_t s = {units, work / units, work % units};
    return s;
}

static inline void sched_unit(const sched_t* s, uint64_t u, uint64_t* base, uint64_t* max)
{
    *base = s->per * u + (u < s->extra ? u : s->extra);
    *max = *base + s->per + (u < s->extra ? 1 : 0);
}

static inline void dyn_init(run_t* r)
{
    if (t_id == 0)
        __atomic_store_n(&r->dyn, (uint64_t)r->threads, __ATOMIC_RELAXED);
    barrier(r);
}

static inline uint64_t dyn_next(run_t* r) { return __sync_fetch_and_add(&r->dyn, 1ull); }

/* phase_edge_pull_bfs.c:86-103 */
static uint64_t find_next_set_bit(const uint64_t* bm, uint64_t start, uint64_t count64)
{
    const uint64_t initialmask = ~((2ull << (start & 63ull)) - 1ull);
    uint64_t cur = start >> 6;
    uint64_t bits = bm[cur] & initialmask;
    while (bits == 0) {
        cur += 1;
        if (cur == count64)
            return UINT64_MAX;
        bits = bm[cur];
    }
    return (cur << 6) + (uint64_t)__builtin_ctzll(bits);
}

/* BFS vector body shared by the dense and Wedge pulls (phase_edge_pull_bfs.c:159-204).
 * Returns 1 to continue, 0 if the visited branch found no unconverged vertex
 * left (phase done), 2 if the visited branch moved last_active. */
static inline int bfs_vector(orc_graph_t* g, const uint64_t* w, uint64_t* changed, uint64_t* last_active)
{
    const uint64_t dst = dst_of(w);
    if (g->props[dst] == UINT64_MAX) {
        uint64_t best = 0;
        int any = 0;
        for (int k = 0; k < 4; ++k) {
            if (!(w[k] & VALID_BIT))
                continue;
            const uint64_t s = w[k] & SRC_MASK;
            if (test_bit(g->snapshot, s)) {
                any = 1;
                if (s > best)
                    best = s; /* _mm_max_pd over the ids, impossible parents = 0 (:178-180) */
            }
        }
        if (!any)
            return 1;
        g->props[dst] = best;
        set_bit(g->active, dst);
        clear_bit(g->unconverged, dst);
        *changed += g->outdeg[dst];
        return 1;
    }
    const uint64_t next = find_next_set_bit(g->unconverged, dst, g->frontier_count);
    if (next >= g->V)
        return 0;
    *last_active = g->index[next];
    return 2;
}

/* phase_edge_pull_bfs.c:109-210 */
static void pull_bfs_dense(run_t* r)
{
    orc_graph_t* g = r->g;
    const sched_t s = sched_make(g->nvec, (uint64_t)r->threads << 5);
    uint64_t changed = 0, last_active = 0;
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        if (last_active > max)
            continue;
        const uint64_t start = last_active > base ? last_active : base;
        for (uint64_t i = start; i < max; ++i) {
            const int rc = bfs_vector(g, &g->vec[i * 4], &changed, &last_active);
            if (rc == 0) {
                r->reduce[t_id] = changed;
                return;
            }
            if (rc == 2)
                i = last_active - 1;
        }
    }
    r->reduce[t_id] = changed;
}

/* phase_edge_pull_bfs.c:212-332 */
static void pull_bfs_wedge(run_t* r)
{
    orc_graph_t* g = r->g;
    const sched_t s = sched_make(g->wedge_count >> 3, (uint64_t)r->threads << 5);
    uint64_t changed = 0, last_active = 0;
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        for (uint64_t i = base; i < max; ++i) {
            const uint64_t fb = i << 3;
            const uint64_t* wf = g->wedge;
            const uint64_t ostart = (wf[fb] | wf[fb + 1] | wf[fb + 2] | wf[fb + 3]) == 0 ? 4 : 0;
            const uint64_t oend = (wf[fb + 4] | wf[fb + 5] | wf[fb + 6] | wf[fb + 7]) == 0 ? 4 : 8;
            for (uint64_t j = ostart; j < oend; ++j) {
                const uint64_t fi = fb + j;
                uint64_t bits = g->wedge[fi];
                if (bits == 0)
                    continue;
                g->wedge[fi] = 0;
                if (((fi + 64ull) << (6ull + LOG2_PRECISION)) < last_active)
                    continue;
                for (; bits != 0; bits &= bits - 1) {
                    const uint64_t vi = (fi << (6ull + LOG2_PRECISION)) +
                                        ((uint64_t)__builtin_ctzll(bits) << LOG2_PRECISION);
                    for (uint64_t k = 0; k < (1ull << LOG2_PRECISION); ++k) {
                        if (vi + k < last_active)
                            continue;
                        const int rc = bfs_vector(g, &g->vec[(vi + k) * 4], &changed, &last_active);
                        if (rc == 0) {
                            r->reduce[t_id] = changed;
                            return;
                        }
                    }
                }
            }
        }
    }
    r->reduce[t_id] = changed;
}

/* ---- min-reduce pulls: CC (double labels) and SSSP (uint64 / FP64 distances) ---- */

/* reduction of the four candidate lanes, per app (phase_edge_pull_cc.c:133-135,
 * phase_edge_pull_sssp.c:136-142) */
static inline uint64_t lane_min_cc(const orc_graph_t* g, const uint64_t* w, uint64_t acc)
{
    double m = as_d(acc);
    for (int k = 0; k < 4; ++k) {
        const double v = (w[k] & VALID_BIT) ? as_d(g->props[w[k] & SRC_MASK]) : INFINITY;
        m = v < m ? v : m;
    }
    return as_u(m);
}

/* _mm_min_epu32 on 64-bit sums: independent minima of the low and high halves */
static inline uint64_t min_epu32(uint64_t a, uint64_t b)
{
    const uint64_t lo = ((a & 0xffffffffull) < (b & 0xffffffffull)) ? (a & 0xffffffffull) : (b & 0xffffffffull);
    const uint64_t hi = ((a >> 32) < (b >> 32)) ? (a >> 32) : (b >> 32);
    return (hi << 32) | lo;
}

static inline uint64_t lane_min_sssp(const orc_graph_t* g, const uint64_t* w, const uint64_t* wt, uint64_t acc)
{
    for (int k = 0; k < 4; ++k) {
        const uint64_t p = (w[k] & VALID_BIT) ? g->props[w[k] & SRC_MASK] : UINT64_MAX;
        const uint64_t adj = (p == UINT64_MAX) ? 0 : wt[k];
        acc = min_epu32(acc, p + adj);
    }
    return acc;
}

static inline uint64_t lane_min_sssp_f64(const orc_graph_t* g, const uint64_t* w, const uint64_t* wt, uint64_t acc)
{
    double m = as_d(acc);
    for (int k = 0; k < 4; ++k) {
        if (!(w[k] & VALID_BIT))
            continue;
        const double v = as_d(g->props[w[k] & SRC_MASK]) + as_d(wt[k]);
        m = v < m ? v : m;
    }
    return as_u(m);
}

enum { MIN_CC, MIN_SSSP, MIN_SSSP_F64 };

static inline uint64_t min_init(int kind) { return kind == MIN_SSSP ? UINT64_MAX : as_u(INFINITY); }

static inline uint64_t min_step(const orc_graph_t* g, int kind, const uint64_t* w, uint64_t acc)
{
    if (kind == MIN_CC)
        return lane_min_cc(g, w, acc);
    if (kind == MIN_SSSP)
        return lane_min_sssp(g, w, w + 4, acc);
    return lane_min_sssp_f64(g, w, w + 4, acc);
}

/* folds one vector's reduced candidates into the destination accumulator
 * (phase_edge_pull_cc.c:135, phase_edge_pull_sssp.c:142) */
static inline uint64_t min_combine(int kind, uint64_t acc, uint64_t cand)
{
    if (kind == MIN_SSSP)
        return min_epu32(cand, acc);
    return as_d(cand) < as_d(acc) ? cand : acc;
}

/* "proposed value differs" test at a destination change: CC compares the bit
 * patterns of min(current, acc) (phase_edge_pull_cc.c:107-113); SSSP writes
 * only when acc < current (phase_edge_pull_sssp.c:112-116). */
static inline int min_propose(int kind, uint64_t cur, uint64_t acc, uint64_t* out)
{
    if (kind == MIN_SSSP) {
        *out = acc < cur ? acc : cur;
        return acc < cur;
    }
    const double c = as_d(cur), a = as_d(acc);
    const double m = c < a ? c : a; /* _mm_min_pd(current, acc) */
    *out = as_u(m);
    return *out != cur;
}

static inline void min_flush(run_t* r, int kind, uint64_t prev, uint64_t acc, uint64_t* changed)
{
    orc_graph_t* g = r->g;
    uint64_t proposed;
    if (min_propose(kind, g->props[prev], acc, &proposed)) {
        g->props[prev] = proposed;
        if (!cond_set_bit(g->active, prev))
            *changed += g->outdeg[prev];
    }
}

static inline void min_unit_end(run_t* r, int kind, uint64_t u, uint64_t prev, uint64_t acc, uint64_t* changed)
{
    orc_graph_t* g = r->g;
    uint64_t proposed;
    const int ch = min_propose(kind, g->props[prev], acc, &proposed);
    r->merge[u].final_vertex_id = prev;
    r->merge[u].final_partial_value = proposed;
    if (ch && !cond_set_bit(g->active, prev))
        *changed += g->outdeg[prev];
}

/* phase_edge_pull_cc.c:53-164, phase_edge_pull_sssp.c:57-169 */
static void pull_min_dense(run_t* r, int kind)
{
    orc_graph_t* g = r->g;
    const uint64_t words = g->weighted ? 8 : 4;
    const sched_t s = sched_make(g->nvec, (uint64_t)r->threads << 5);
    uint64_t changed = 0;
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        if (base == max)
            continue; /* deviation: see file header */
        uint64_t acc = min_init(kind), prev = UINT64_MAX;
        for (uint64_t i = base; i < max; ++i) {
            const uint64_t* w = &g->vec[i * words];
            /* the gather precedes the flush of the previous destination
             * (phase_edge_pull_cc.c:99 before :105-128), so a destination does
             * not yet see its predecessor's update of this pass */
            const uint64_t cand = min_step(g, kind, w, min_init(kind));
            const uint64_t d = dst_of(w);
            if (prev < d) {
                min_flush(r, kind, prev, acc, &changed);
                acc = min_init(kind);
            }
            prev = d;
            acc = min_combine(kind, acc, cand);
        }
        min_unit_end(r, kind, u, prev, acc, &changed);
    }
    r->reduce[t_id] = changed;
}

/* phase_edge_pull_cc.c:166-297, phase_edge_pull_sssp.c:171-306 */
static void pull_min_wedge(run_t* r, int kind)
{
    orc_graph_t* g = r->g;
    const uint64_t words = g->weighted ? 8 : 4;
    const sched_t s = sched_make(g->wedge_count >> 3, (uint64_t)r->threads << 5);
    uint64_t changed = 0;
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        uint64_t acc = min_init(kind), prev = UINT64_MAX;
        for (uint64_t i = base; i < max; ++i) {
            const uint64_t fb = i << 3;
            const uint64_t* wf = g->wedge;
            const uint64_t ostart = (wf[fb] | wf[fb + 1] | wf[fb + 2] | wf[fb + 3]) == 0 ? 4 : 0;
            const uint64_t oend = (wf[fb + 4] | wf[fb + 5] | wf[fb + 6] | wf[fb + 7]) == 0 ? 4 : 8;
            for (uint64_t j = ostart; j < oend; ++j) {
                const uint64_t fi = fb + j;
                uint64_t bits = g->wedge[fi];
                if (bits == 0)
                    continue;
                g->wedge[fi] = 0;
                for (; bits != 0; bits &= bits - 1) {
                    const uint64_t vi = (fi << (6ull + LOG2_PRECISION)) +
                                        ((uint64_t)__builtin_ctzll(bits) << LOG2_PRECISION);
                    for (uint64_t k = 0; k < (1ull << LOG2_PRECISION); ++k) {
                        const uint64_t* w = &g->vec[(vi + k) * words];
                        const uint64_t cand = min_step(g, kind, w, min_init(kind)); /* gather first */
                        const uint64_t d = dst_of(w);
                        if (prev < d) {
                            min_flush(r, kind, prev, acc, &changed);
                            acc = min_init(kind);
                        }
                        prev = d;
                        acc = min_combine(kind, acc, cand);
                    }
                }
            }
        }
        if (prev != UINT64_MAX)
            min_unit_end(r, kind, u, prev, acc, &changed);
    }
    r->reduce[t_id] = changed;
}

/* phases.c:54-69: idempotent merge (min) of the unit-boundary partials */
static void merge_idempotent(run_t* r, int kind)
{
    orc_graph_t* g = r->g;
    const uint64_t n = (uint64_t)r->threads * 32ull;
    for (uint64_t i = 0; i < n; ++i) {
        if (r->merge[i].final_vertex_id & VALID_BIT)
            continue;
        const uint64_t v = r->merge[i].final_vertex_id;
        const uint64_t a = g->props[v], b = r->merge[i].final_partial_value;
        if (kind == MIN_SSSP)
            g->props[v] = a < b ? a : b; /* execution_sssp.c:63-66 */
        else
            g->props[v] = as_d(a) < as_d(b) ? a : b; /* execution_cc.c:62-65 */
        r->merge[i].final_vertex_id = VALID_BIT;
    }
}

/* wedge.c:37-46 */
static inline void wedge_activate(orc_graph_t* g, uint64_t v)
{
    for (uint64_t i = g->csri_index[v]; i < g->csri_index[v + 1]; ++i) {
        const uint64_t e = g->csri_edges[i];
        uint8_t* a = &((uint8_t*)g->wedge)[e >> 3];
        const uint8_t m = (uint8_t)(1u << (e & 7));
        if (!(__atomic_load_n(a, __ATOMIC_RELAXED) & m))
            __atomic_fetch_or(a, m, __ATOMIC_RELAXED);
    }
}

/* wedge.c:63-155 */
static void wedge_generate(run_t* r)
{
    orc_graph_t* g = r->g;
    const sched_t s = sched_make(g->frontier_count >> 3, (uint64_t)r->threads << 5);
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        for (uint64_t i = base; i < max; ++i) {
            for (uint64_t j = 0; j < 8; ++j) {
                const uint64_t wi = (i << 3) + j;
                for (uint64_t bits = g->active[wi]; bits != 0; bits &= bits - 1)
                    wedge_activate(g, (wi << 6) + (uint64_t)__builtin_ctzll(bits));
            }
        }
    }
}

/* parutilMemorySet inside a parallel region: each thread clears its chunk */
static void par_memset(run_t* r, void* buf, int val, size_t bytes)
{
    const uint64_t n = (uint64_t)r->threads, id = (uint64_t)t_id;
    const uint64_t per = bytes / n, extra = bytes % n;
    const uint64_t start = per * id + (id < extra ? id : extra);
    memset((uint8_t*)buf + start, val, per + (id < extra ? 1 : 0));
    barrier(r);
}

/* execution_cc.c:260-271: clear only the non-zero 256-bit groups */
static void sparse_clear_active(run_t* r)
{
    orc_graph_t* g = r->g;
    const uint64_t groups = g->frontier_count >> 2;
    const uint64_t n = (uint64_t)r->threads, id = (uint64_t)t_id;
    const uint64_t per = groups / n, extra = groups % n;
    const uint64_t lo = per * id + (id < extra ? id : extra), hi = lo + per + (id < extra ? 1 : 0);
    for (uint64_t i = lo; i < hi; ++i) {
        uint64_t* a = &g->active[i << 2];
        if (a[0] | a[1] | a[2] | a[3])
            a[0] = a[1] = a[2] = a[3] = 0;
    }
}

static uint64_t combine_u64(run_t* r) /* phases.c:26-35 */
{
    uint64_t v = 0;
    for (int i = 0; i < r->threads; ++i)
        v += r->reduce[i];
    return v;
}

static double combine_f64(run_t* r) /* phases.c:37-46 */
{
    double v = 0.0;
    for (int i = 0; i < r->threads; ++i)
        v += as_d(r->reduce[i]);
    return v;
}

/* ---- app init (execution_*_initialize) ---- */
static void init_static_range(run_t* r, uint64_t* lo, uint64_t* hi)
{
    const uint64_t n = (uint64_t)r->threads, id = (uint64_t)t_id, V = r->g->V;
    const uint64_t per = V / n, extra = V % n;
    *lo = per * id + (id < extra ? id : extra);
    *hi = *lo + per + (id < extra ? 1 : 0);
}

/* ---- drivers ---- */

/* execution_bfs.c:84-118 + :122-365 */
static void drive_bfs(run_t* r)
{
    orc_graph_t* g = r->g;
    uint64_t lo, hi;
    init_static_range(r, &lo, &hi);
    for (uint64_t v = lo; v < hi; ++v) {
        if (g->index[v] == UINT64_MAX)
            clear_bit(g->unconverged, v);
        g->props[v] = UINT64_MAX;
    }
    barrier(r);
    if (t_id == 0) {
        set_bit(g->snapshot, r->p.root);
        clear_bit(g->unconverged, r->p.root);
        wedge_activate(g, r->p.root);
    }
    barrier(r);

    const uint64_t threshold = (g->E * r->p.threshold_pct) / 100ull;
    uint64_t active = g->outdeg[r->p.root];
    uint64_t ctr = 0, ctr_wedge = 0;
    double t0 = 0;
    while (1) {
        const bool dense = active > threshold;
        ++ctr;
        if (t_id == 0)
            t0 = now_ms();
        if (dense)
            pull_bfs_dense(r);
        else {
            ++ctr_wedge;
            pull_bfs_wedge(r);
        }
        barrier(r);
        if (t_id == 0) {
            const double dt = now_ms() - t0;
            if (dense)
                r->stats.pull_ms_nowedge += dt;
            else
                r->stats.pull_ms_wedge += dt;
        }
        active = combine_u64(r);
        if (active == 0)
            break;
        barrier(r);
        if (t_id == 0)
            t0 = now_ms();
        if (active <= threshold)
            wedge_generate(r);
        barrier(r);
        if (t_id == 0) {
            r->stats.wedge_ms += now_ms() - t0;
            t0 = now_ms();
        }
        barrier(r);
        if (t_id == 0) {
            uint64_t* t = g->active;
            g->active = g->snapshot;
            g->snapshot = t;
        }
        barrier(r);
        par_memset(r, g->active, 0, g->frontier_count << 3);
        barrier(r);
        if (t_id == 0) {
            const double dt = now_ms() - t0;
            if (dense)
                r->stats.pull_ms_nowedge += dt;
            else
                r->stats.pull_ms_wedge += dt;
        }
    }
    if (t_id == 0) {
        r->stats.iterations = ctr;
        r->stats.wedge_iterations = ctr_wedge;
    }
}

/* execution_cc.c:69-325 and execution_sssp.c:70-334 */
static void drive_min(run_t* r, int kind)
{
    orc_graph_t* g = r->g;
    uint64_t lo, hi;
    init_static_range(r, &lo, &hi);
    const bool is_cc = kind == MIN_CC;
    for (uint64_t v = lo; v < hi; ++v)
        g->props[v] = is_cc ? as_u((double)v) : (kind == MIN_SSSP ? UINT64_MAX : as_u(INFINITY));
    barrier(r);
    if (!is_cc && t_id == 0) {
        g->props[r->p.root] = kind == MIN_SSSP ? 0ull : as_u(0.0);
        wedge_activate(g, r->p.root);
    }
    barrier(r);

    const uint64_t threshold = (g->E * r->p.threshold_pct) / 100ull;
    uint64_t active = is_cc ? g->E : g->outdeg[r->p.root];
    uint64_t ctr = 0, ctr_wedge = 0;
    double t0 = 0;
    while (1) {
        const bool dense = (active > threshold) || (is_cc && ctr == 0);
        ++ctr;
        if (t_id == 0)
            t0 = now_ms();
        if (dense)
            pull_min_dense(r, kind);
        else {
            ++ctr_wedge;
            pull_min_wedge(r, kind);
        }
        barrier(r);
        if (t_id == 0)
            merge_idempotent(r, kind);
        barrier(r);
        if (t_id == 0) {
            const double dt = now_ms() - t0;
            if (dense)
                r->stats.pull_ms_nowedge += dt;
            else
                r->stats.pull_ms_wedge += dt;
        }
        active = combine_u64(r);
        if (active == 0)
            break;
        barrier(r);
        if (t_id == 0)
            t0 = now_ms();
        if (active <= threshold) {
            wedge_generate(r);
            barrier(r);
            sparse_clear_active(r);
        } else {
            par_memset(r, g->active, 0, g->frontier_count << 3);
        }
        barrier(r);
        if (t_id == 0)
            r->stats.wedge_ms += now_ms() - t0;
        barrier(r);
    }
    if (t_id == 0) {
        r->stats.iterations = ctr;
        r->stats.wedge_iterations = ctr_wedge;
    }
}

/* phase_edge_pull_pr.c:28-116 */
static void pull_pr(run_t* r)
{
    orc_graph_t* g = r->g;
    const sched_t s = sched_make(g->nvec, (uint64_t)r->threads << 5);
    double total = 0.0; /* lane 0 of __m128d total_rank (both lanes are equal) */
    dyn_init(r);
    for (uint64_t u = (uint64_t)t_id; u < s.units; u = dyn_next(r)) {
        uint64_t base, max;
        sched_unit(&s, u, &base, &max);
        double a[4] = {0, 0, 0, 0};
        uint64_t prev = dst_of(&g->vec[base * 4]);
        r->merge[u].initial_vertex_id = prev;
        for (uint64_t i = base; i < max; ++i) {
            const uint64_t* w = &g->vec[i * 4];
            double p[4];
            for (int k = 0; k < 4; ++k)
                p[k] = (w[k] & VALID_BIT) ? as_d(g->props[w[k] & SRC_MASK]) : 0.0;
            const uint64_t d = dst_of(w);
            if (prev < d) {
                /* hadd: [a0+a1, a0+a1, a2+a3, a2+a3]; low + high lanes */
                const double part = (a[0] + a[1]) + (a[2] + a[3]);
                g->acc[prev] = as_u(part);
                total += part;
                a[0] = a[1] = a[2] = a[3] = 0.0;
            }
            prev = d;
            for (int k = 0; k < 4; ++k)
                a[k] += p[k];
        }
        r->merge[u].final_vertex_id = prev;
        const double part = (a[0] + a[1]) + (a[2] + a[3]);
        r->merge[u].final_partial_value = as_u(part);
        total += part;
    }
    r->reduce[t_id] = as_u(total);
}

/* phases.c:71-114: ordered (non-idempotent) merge of unit-boundary partial sums */
static void merge_ordered_sum(run_t* r)
{
    orc_graph_t* g = r->g;
    const uint64_t n = (uint64_t)r->threads * 32ull;
    double proposed = 0.0;
    uint64_t last = UINT64_MAX;
    for (uint64_t i = 0; i < n; ++i) {
        mergeaccum_t* m = &r->merge[i];
        if (m->final_vertex_id & VALID_BIT)
            continue;
        if (last == UINT64_MAX) {
            last = m->final_vertex_id;
            proposed = as_d(m->final_partial_value);
        } else if (last == m->final_vertex_id) {
            proposed = proposed + as_d(m->final_partial_value);
        } else {
            if (last == m->initial_vertex_id)
                proposed = proposed + as_d(g->acc[last]);
            g->acc[last] = as_u(proposed);
            last = m->final_vertex_id;
            proposed = as_d(m->final_partial_value);
        }
        m->final_vertex_id = VALID_BIT;
    }
    if (last != UINT64_MAX)
        g->acc[last] = as_u(proposed);
}

/* phase_vertex_pr.c:26-77 */
static void vertex_pr(run_t* r)
{
    orc_graph_t* g = r->g;
    const double N = (double)g->V;
    const double d = r->damping;
    const double omd = (1.0 - d) / N;
    const double total = combine_f64(r);
    const double corr = (1.0 - total) / N;
    const uint64_t iters = (g->V >> 2) + ((g->V & 3ull) ? 1 : 0);
    const uint64_t n = (uint64_t)r->threads, id = (uint64_t)t_id;
    const uint64_t per = iters / n, extra = iters % n;
    const uint64_t lo = per * id + (id < extra ? id : extra), hi = lo + per + (id < extra ? 1 : 0);
    for (uint64_t i = lo; i < hi; ++i) {
        for (uint64_t k = 0; k < 4; ++k) {
            const uint64_t v = (i << 2) + k;
            const double od = g->outdeg[v] == 0 ? N : as_d(g->outdeg[v]);
            const double a = as_d(g->acc[v]);
            g->props[v] = as_u(((a + corr) * d + omd) / od);
        }
    }
}

/* execution_pr.c:380-392 + :396-486 */
static void drive_pr(run_t* r)
{
    orc_graph_t* g = r->g;
    const double N = (double)g->V;
    uint64_t lo, hi;
    init_static_range(r, &lo, &hi);
    for (uint64_t v = lo; v < hi; ++v) {
        const double od = (double)g->outdeg[v];
        g->outdeg[v] = as_u(od);
        g->acc[v] = as_u(0.0);
        g->props[v] = as_u((1.0 / N) / (od == 0.0 ? N : od));
    }
    barrier(r);
    double t0 = 0;
    uint64_t ctr;
    for (ctr = 0; ctr < r->p.iterations; ++ctr) {
        if (t_id == 0)
            t0 = now_ms();
        pull_pr(r);
        barrier(r);
        if (t_id == 0)
            merge_ordered_sum(r);
        barrier(r);
        vertex_pr(r);
        barrier(r);
        if (t_id == 0)
            r->stats.pull_ms_nowedge += now_ms() - t0;
    }
    if (t_id == 0) {
        r->stats.iterations = ctr;
        r->stats.wedge_iterations = 0;
    }
}

typedef struct {
    run_t* r;
    int id;
} worker_t;

static void* worker_main(void* p)
{
    worker_t* w = (worker_t*)p;
    run_t* r = w->r;
    t_id = w->id;
    switch (r->app) {
    case ORC_BFS:
        drive_bfs(r);
        break;
    case ORC_CC:
        drive_min(r, MIN_CC);
        break;
    case ORC_SSSP:
        drive_min(r, r->p.weight_kind == ORC_WEIGHTS_F64 ? MIN_SSSP_F64 : MIN_SSSP);
        break;
    case ORC_PR:
        drive_pr(r);
        break;
    }
    return NULL;
}

int orc_run(orc_graph_t* g, int app, const orc_params_t* p, orc_stats_t* stats)
{
    if (!g || !p || app < 0 || app > 3)
        return ORC_ERR_ARG;
    if ((app == ORC_SSSP) != (g->weighted != 0))
        return ORC_ERR_ARG;
    run_t* r = (run_t*)calloc(1, sizeof(run_t));
    if (!r)
        return ORC_ERR_OOM;
    r->g = g;
    r->p = *p;
    if (r->p.root >= g->V)
        r->p.root = 0; /* main.c:81-85 */
    r->app = app;
    r->threads = p->threads > 0 ? p->threads : orc_online_cores();
    r->damping = p->damping > 0 ? p->damping : 0.875;
    r->reduce = (uint64_t*)calloc((size_t)r->threads + 8, 8);
    r->merge = (mergeaccum_t*)calloc((size_t)r->threads * 32, sizeof(mergeaccum_t));
    if (!r->reduce || !r->merge) {
        free(r->reduce);
        free(r->merge);
        free(r);
        return ORC_ERR_OOM;
    }
    for (int i = 0; i < r->threads * 32; ++i) {
        r->merge[i].initial_vertex_id = UINT64_MAX;
        r->merge[i].final_vertex_id = UINT64_MAX;
    }
    /* fresh frontiers for every run (graphdata.c:845-892 zero / 0xff fill) */
    memset(g->wedge, 0, g->wedge_count * 8);
    memset(g->active, 0, g->frontier_count * 8);
    memset(g->snapshot, 0, g->frontier_count * 8);
    memset(g->unconverged, 0xff, g->frontier_count * 8);
    if (g->outdeg_f64) { /* a previous PageRank run left double out-degrees */
        for (uint64_t v = 0; v < g->V; ++v)
            g->outdeg[v] = (uint64_t)as_d(g->outdeg[v]);
        g->outdeg_f64 = 0;
    }
    if (app == ORC_PR)
        g->outdeg_f64 = 1;
    pthread_barrier_init(&r->bar, NULL, (unsigned)r->threads);
    pthread_t* th = (pthread_t*)calloc((size_t)r->threads, sizeof(pthread_t));
    worker_t* ws = (worker_t*)calloc((size_t)r->threads, sizeof(worker_t));
    for (int i = 1; i < r->threads; ++i) {
        ws[i].r = r;
        ws[i].id = i;
        pthread_create(&th[i], NULL, worker_main, &ws[i]);
    }
    ws[0].r = r;
    ws[0].id = 0;
    worker_main(&ws[0]);
    for (int i = 1; i < r->threads; ++i)
        pthread_join(th[i], NULL);
    pthread_barrier_destroy(&r->bar);
    r->stats.running_ms = r->stats.pull_ms_nowedge + r->stats.pull_ms_wedge + r->stats.wedge_ms;
    if (stats)
        *stats = r->stats;
    free(th);
    free(ws);
    free(r->reduce);
    free(r->merge);
    free(r);
    return ORC_OK;
}
