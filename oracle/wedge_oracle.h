/*
 * ORACLE -- test infrastructure, not product code.
 *
 * A portable-C restatement of the reference's pull-only edge-pull engine
 * (stanford-mast/Wedge) plus the project's synthetic graph generators.
 * Only tests/, the smoke check in __graft_entry__.py and bench.py's CPU
 * baseline legs may load it; the CUDA engine never calls it.
 *
 * Parity of this restatement is pinned against the reference itself, built
 * here from its own sources (oracle/Makefile `ref`), through the golden
 * fixtures in tests/golden/.
 */
#ifndef WEDGE_ORACLE_H
#define WEDGE_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_BFS = 0, ORC_CC = 1, ORC_PR = 2, ORC_SSSP = 3 };
enum { ORC_WEIGHTS_NONE = -1, ORC_WEIGHTS_U64 = 0, ORC_WEIGHTS_F64 = 1 };
enum {
    ORC_OK = 0,
    ORC_ERR_IO = -1,
    ORC_ERR_FORMAT = -2,
    ORC_ERR_OOM = -3,
    ORC_ERR_ARG = -6
};

typedef struct orc_graph orc_graph_t;

typedef struct orc_params {
    uint64_t root;           /* -r, source/cmdline.c:329-448, default 0 */
    uint64_t threshold_pct;  /* -t, default 20 (include/cmdline.h:30) */
    uint64_t iterations;     /* -N, PageRank only, default 1 */
    double damping;          /* include/constants.h:39 hard-codes 0.875 */
    int32_t threads;         /* -n; 0 = all online cores */
    int32_t weight_kind;     /* SSSP: ORC_WEIGHTS_U64 (reference) or ORC_WEIGHTS_F64 (restatement only) */
} orc_params_t;

typedef struct orc_stats {
    uint64_t iterations;        /* total_iterations_executed */
    uint64_t wedge_iterations;  /* total_wedge_iterations_executed */
    double running_ms;          /* pull + activation, source/main.c:154-155 */
    double pull_ms_nowedge;
    double pull_ms_wedge;
    double wedge_ms;
} orc_stats_t;

/* ---- generators (project specification; the CUDA generator matches them bit-for-bit) ---- */
uint64_t orc_mix64(uint64_t z);
uint64_t orc_draw(uint64_t seed, uint64_t item, uint64_t word);
void orc_rmat_thresholds(double a, double b, double c, uint64_t out[3]);
void orc_rmat(uint32_t scale, double a, double b, double c, uint64_t seed, uint64_t first,
              uint64_t count, uint32_t* src, uint32_t* dst, int threads);
uint64_t orc_grid_edge_count(uint64_t side, double long_range_frac);
void orc_grid(uint64_t side, double long_range_frac, uint64_t seed, uint32_t* src, uint32_t* dst);
uint64_t orc_weight_u64(uint64_t s, uint64_t d);
double orc_weight_f64(uint64_t s, uint64_t d);
void orc_weights(uint64_t E, const uint32_t* src, const uint32_t* dst, int kind, uint64_t* out);
/* stable sort of an edge list into (dst, src) order; returns ORC_OK */
int orc_sort_edges(uint64_t V, uint64_t E, uint32_t* src, uint32_t* dst, int threads);
/* append the reverse of every edge (E -> 2E entries; arrays must hold 2E) */
void orc_symmetrise(uint64_t E, uint32_t* src, uint32_t* dst);
/* Wedge binary edge-list file, README.md:42-50 / graphdata.c:589-642 */
int orc_write_file(const char* path, uint64_t V, uint64_t E, const uint32_t* src, const uint32_t* dst,
                   const uint64_t* weights);

/* ---- engine (restates graphdata.c, wedge.c, phases.c, phase_*.c, execution_*.c) ---- */
int orc_load_file(const char* path, int app, int threads, orc_graph_t** out);
int orc_build(uint64_t V, uint64_t E, const uint32_t* src, const uint32_t* dst, const uint64_t* weights,
              int app, int threads, orc_graph_t** out);
int orc_run(orc_graph_t* g, int app, const orc_params_t* p, orc_stats_t* stats);
uint64_t orc_num_vertices(const orc_graph_t* g);
uint64_t orc_num_edges(const orc_graph_t* g);
uint64_t orc_num_edge_vectors(const orc_graph_t* g);
const uint64_t* orc_props(const orc_graph_t* g);     /* graph_vertex_props, V words */
const uint64_t* orc_outdegrees(const orc_graph_t* g); /* graph_vertex_outdegrees, V words */
/* the edge-vector words the reference would hold in graph_edges_gather_list_bufs_numa[0] */
const uint64_t* orc_edge_vectors(const orc_graph_t* g, uint64_t* words);
void orc_free(orc_graph_t* g);
int orc_online_cores(void);

#ifdef __cplusplus
}
#endif
#endif
