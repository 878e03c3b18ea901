/*
 * wedge_cuda.h -- C ABI of the GB300 (sm_103a) edge-pull engine.
 *
 * This is the drop-in boundary for Wedge's pull-only edge-pull path.  A C host
 * that today runs
 *     application_select -> graph_data_read_from_file ->
 *     graph_data_initialize_data_structures -> execution_impl_* ->
 *     execution_get_vertex_prop_string_*
 * calls, in the same order,
 *     wedge_cuda_load_graph -> wedge_cuda_run -> wedge_cuda_read_results.
 *
 * Conventions
 *  - Plain C types only; no CUDA or framework types cross this boundary.
 *  - Every function returns WEDGE_OK (0) or a negative WEDGE_ERR_* status.
 *  - One host thread per graph handle.  The device owns all graph and
 *    property memory; the host receives copies.
 *  - Vertex ids are < 2^32 - 1 on the device (the reference allows 48 bits,
 *    graphdata.c:212-243); larger graphs are rejected with WEDGE_ERR_FORMAT.
 *  - Properties come back in the reference's own representation, one 64-bit
 *    word per vertex as in graph_vertex_props (include/graphdata.h:54):
 *      BFS  uint64 parent, UINT64_MAX = unreached   (execution_bfs.c:69-73)
 *      CC   double label                             (execution_cc.c:47-51)
 *      PR   double rank / outdegree'                 (execution_pr.c:31-35)
 *      SSSP uint64 distance, UINT64_MAX = unreached  (execution_sssp.c:48-52)
 *           or double distance for FP64 weights (no reference counterpart).
 */
#ifndef WEDGE_CUDA_H
#define WEDGE_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WEDGE_CUDA_ABI_VERSION 2

/* application ids; names and aliases as in source/application.c:49-68 */
enum wedge_app {
    WEDGE_APP_BFS = 0,
    WEDGE_APP_CC = 1,
    WEDGE_APP_PR = 2,
    WEDGE_APP_SSSP = 3
};

enum wedge_status {
    WEDGE_OK = 0,
    WEDGE_ERR_IO = -1,             /* file missing, short read (graphdata.c:960-965) */
    WEDGE_ERR_FORMAT = -2,         /* size mismatch, unsorted dst, id out of range (graphdata.c:968-979) */
    WEDGE_ERR_OOM = -3,
    WEDGE_ERR_CUDA = -4,
    WEDGE_ERR_NOT_CONVERGED = -5,  /* iteration cap reached before the frontier emptied */
    WEDGE_ERR_ARG = -6,
    WEDGE_ERR_UNSUPPORTED = -7
};

/* how the third word of a weighted edge record is read */
enum wedge_weights {
    WEDGE_WEIGHTS_NONE = 0,
    WEDGE_WEIGHTS_U64 = 1, /* reference behaviour (phase_edge_pull_sssp.c:93,137) */
    WEDGE_WEIGHTS_F64 = 2  /* IEEE double weights, double min-plus */
};

enum wedge_precision {
    WEDGE_PREC_FP64 = 0,  /* reference arithmetic (PageRank) */
    WEDGE_PREC_FP32C = 1  /* FP32 ranks, per-destination two-sum compensated sums, FP64 global terms */
};

/* how each iteration chooses its pull strategy (enum wedge_mode) */
enum wedge_sched {
    WEDGE_SCHED_PLAIN = 0,     /* fixed threshold: dense iff active out-edge mass > t% of |E| (execution_bfs.c:132,141) */
    WEDGE_SCHED_DENSE = 1,     /* always dense */
    WEDGE_SCHED_WEDGE = 2,     /* Wedge whenever the frontier allows it */
    WEDGE_SCHED_FILTERED = 3,  /* source-filtered sweep whenever the frontier allows it */
    WEDGE_SCHED_LEARNED = 4,   /* the scheduler network set by wedge_cuda_set_scheduler, evaluated on the
                                  device after every pull; the plain rule where its features leave the
                                  trained range or its predicted gain is below the network's margin */
    WEDGE_SCHED_PROBE = 5      /* plain, except that iteration probe_iter uses probe_mode (timing data) */
};

/* pull strategy of one iteration (no counterpart in the reference beyond dense / Wedge) */
enum wedge_mode {
    WEDGE_MODE_DENSE = 0,    /* every tile (perform_edge_pull_phase_*) */
    WEDGE_MODE_WEDGE = 1,    /* the tiles of the Wedge frontier (*_with_wedge_frontier) */
    WEDGE_MODE_FILTERED = 2  /* every tile, gathering only from sources the previous pull changed
                                (CC/SSSP; BFS runs it as dense, whose gathers are frontier bits) */
};

/* single phases, for hosts that keep the reference's own driver loop (include/phases.h:58-88, wedge.h:24-27) */
enum wedge_phase {
    WEDGE_PHASE_INIT = 0,          /* execution_initialize_* */
    WEDGE_PHASE_PULL_DENSE = 1,    /* perform_edge_pull_phase_{bfs,cc,pr,sssp} */
    WEDGE_PHASE_PULL_WEDGE = 2,    /* perform_edge_pull_phase_*_with_wedge_frontier */
    WEDGE_PHASE_VERTEX_PR = 3,     /* edge_pull_op_merge_with_merge_buffer + perform_vertex_phase_pr */
    WEDGE_PHASE_WEDGE_BUILD = 4,   /* wedge_generate_frontier */
    WEDGE_PHASE_ADVANCE = 5        /* frontier swap / clear between iterations (execution_bfs.c:320-338) */
};

#define WEDGE_FLAG_GRAPH 1u   /* run the traversal as one CUDA graph looping on a device convergence flag */
#define WEDGE_FLAG_TIMING 2u  /* record per-phase CUDA events (Pull/Wedge times of the statistics block) */

typedef struct wedge_params {
    uint64_t root;            /* -r, default 0 (include/cmdline.h:29) */
    uint32_t threshold_pct;   /* -t, default 20 (include/cmdline.h:30) */
    uint32_t num_iterations;  /* -N, PageRank iterations, default 1 (include/cmdline.h:28) */
    double damping;           /* PageRank damping; 0 selects the reference's 0.875 (include/constants.h:39) */
    int32_t precision;        /* enum wedge_precision (PageRank only) */
    int32_t sched;            /* enum wedge_sched */
    uint32_t max_iterations;  /* cap for BFS/CC/SSSP; 0 = |V| + 1 */
    uint32_t flags;           /* WEDGE_FLAG_* */
    uint32_t probe_iter;      /* WEDGE_SCHED_PROBE: the iteration whose strategy is forced */
    int32_t probe_mode;       /* WEDGE_SCHED_PROBE: its enum wedge_mode */
} wedge_params_t;

/* EXECUTION STATISTICS block of source/main.c:153-182, plus device counters */
typedef struct wedge_stats {
    uint64_t iterations;          /* Total Iterations */
    uint64_t wedge_iterations;    /* Iterations with Wedge */
    double running_ms;            /* Running Time: whole traversal on the device */
    double pull_ms_dense;         /* No Frontier Pull Time (needs WEDGE_FLAG_TIMING) */
    double pull_ms_wedge;         /* Frontier Pull Time (needs WEDGE_FLAG_TIMING) */
    double wedge_ms;              /* Wedge Time (needs WEDGE_FLAG_TIMING) */
    double vertex_ms;             /* PageRank vertex phase (needs WEDGE_FLAG_TIMING) */
    uint64_t edges_scanned;       /* in-edges read by the pulls, summed over iterations */
    uint64_t tiles_scanned;       /* 128-edge tiles visited by the pulls */
    uint64_t dsts_scanned;        /* destinations with in-edges in the visited tiles */
    uint64_t vertices_activated;  /* vertices whose property changed (BFS: newly visited) */
    uint64_t pull_launches;       /* edge-pull kernel launches */
    uint64_t kernel_launches;     /* all kernel launches of the run */
    double pr_sum;                /* PageRank Sum (execution_pr.c:63-71); 0 for other apps */
} wedge_stats_t;

/* scheduler network: WEDGE_SCHED_FEATURES inputs -> 64 -> 64 -> 3 (ReLU, FP32); the outputs are
 * predicted log2 costs (microseconds) of the three enum wedge_mode strategies */
#define WEDGE_SCHED_FEATURES 16
#define WEDGE_SCHED_HIDDEN 64
#define WEDGE_SCHED_OUTPUTS 3
/* float layout of a network blob (WEDGE_SCHED_BLOB floats):
 *   mu[16] sd[16]      feature standardisation x' = (x - mu) / sd
 *   lo[16] hi[16]      trained feature range (outside it: the plain rule)
 *   W1[64][16] b1[64] W2[64][64] b2[64] W3[3][64] b3[3]
 *   margin             least predicted log2 gain over the plain choice to take the network's choice
 * The trainable part (W1..b3, WEDGE_SCHED_PARAMS floats) starts at WEDGE_SCHED_PARAM_OFFSET. */
#define WEDGE_SCHED_PARAM_OFFSET 64
#define WEDGE_SCHED_PARAMS (64 * 16 + 64 + 64 * 64 + 64 + 3 * 64 + 3)
#define WEDGE_SCHED_BLOB (WEDGE_SCHED_PARAM_OFFSET + WEDGE_SCHED_PARAMS + 1)

/* one iteration of a traversal: the ITERATION_STATS record the reference prints to stderr
 * (execution_bfs.c:227-232: active edges, used Wedge, pull ms, Wedge ms) plus device counters */
typedef struct wedge_iteration_record {
    uint64_t active_edges;        /* changed-edge mass that chose this iteration's pull */
    uint32_t used_wedge;          /* 1 if the pull used the Wedge frontier */
    uint32_t iteration;
    double pull_ms;               /* pull time, or -1 unless the run had WEDGE_FLAG_TIMING */
    double wedge_ms;              /* Wedge-frontier build time after the pull, or -1 */
    uint64_t changed_mass;        /* changed-edge mass the pull produced */
    uint64_t edges_scanned;
    uint64_t tiles_scanned;
    uint64_t dsts_scanned;
    uint64_t vertices_activated;
    uint32_t mode;                /* enum wedge_mode of the pull */
    uint32_t learned;             /* 1 if the scheduler network chose it */
    float features[WEDGE_SCHED_FEATURES]; /* the scheduler features the mode was chosen on (iterations >= 1) */
} wedge_iteration_record_t;

typedef struct wedge_graph wedge_graph_t;

/* ---------------------------------------------------------------- loading */

/* graph_data_read_from_file (graphdata.c:946-1133) + graph_data_initialize_data_structures
 * (graphdata.c:648-942).  The file is header {uint64 V, uint64 E} followed by E records
 * {uint64 src, uint64 dst} -- or {src, dst, weight} when app == WEDGE_APP_SSSP
 * (application.c:171) -- grouped by ascending dst.  The size is checked exactly. */
int wedge_cuda_load_graph(const char* path, int app, wedge_graph_t** out);

/* as wedge_cuda_load_graph, choosing how SSSP weights are read (enum wedge_weights) */
int wedge_cuda_load_graph_ex(const char* path, int app, int weight_kind, wedge_graph_t** out);

/* the same file format, already in host memory (bytes = whole file image) */
int wedge_cuda_load_graph_image(const void* image, uint64_t bytes, int app, int weight_kind, wedge_graph_t** out);

/* host edge arrays grouped by ascending dst (the file's records without the header);
 * weights may be NULL (weight_kind NONE) or hold raw 64-bit words */
int wedge_cuda_load_edges(uint64_t num_vertices, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                          const uint64_t* weights, int weight_kind, wedge_graph_t** out);

/* the reference's in-memory edge-vector list (graphdata.c:212-243; one vector = 4 words
 * valid|dst-slice|src48, followed by 4 weight words when weighted), as a host would pass it
 * to perform_edge_pull_phase_* (include/phases.h:58-60) */
int wedge_cuda_load_edge_vectors(uint64_t num_vertices, const uint64_t* vectors, uint64_t num_vectors,
                                 int weighted, int weight_kind, wedge_graph_t** out);

/* synthetic inputs generated on the device (bit-identical to the CPU generators):
 * R-MAT with quadrant probabilities a,b,c; symmetrise adds every reverse edge */
int wedge_cuda_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                             int symmetrise, int weight_kind, wedge_graph_t** out);
/* side x side 4-neighbour grid, both directions, plus floor(frac * 4*side*(side-1)) random directed pairs */
int wedge_cuda_generate_grid(uint32_t side, double long_range_frac, uint64_t seed, int weight_kind,
                             wedge_graph_t** out);
/* The same generators' edge lists, sorted by (dst, src) as the reference's file format
 * orders them (README.md:42-50), into host arrays of `capacity` entries (the wedge-gen
 * writer).  With src == NULL only *V and *E are returned. */
int wedge_cuda_rmat_edge_list(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                              int symmetrise, uint64_t* V, uint64_t* E, uint32_t* src, uint32_t* dst,
                              uint64_t capacity);
int wedge_cuda_grid_edge_list(uint32_t side, double long_range_frac, uint64_t seed, uint64_t* V, uint64_t* E,
                              uint32_t* src, uint32_t* dst, uint64_t capacity);

/* ---------------------------------------------------------------- running */

/* execution_initialize_* + execution_impl_{bfs,cc,pr,sssp} (execution.h:107-129): the whole
 * traversal on the device; stats may be NULL.  Properties stay on the device. */
int wedge_cuda_run(wedge_graph_t* g, int app, const wedge_params_t* params, wedge_stats_t* stats);

/* one phase (enum wedge_phase) of the reference's driver loop, for hosts that sequence phases
 * themselves.  *active_mass receives the reduced changed-edge mass after a pull
 * (phase_op_combine_global_var_from_buf, phases.c:26-35) and may be NULL. */
int wedge_cuda_run_phase(wedge_graph_t* g, int app, int phase, const wedge_params_t* params,
                         uint64_t* active_mass);

/* Asynchronous forms (no counterpart in the reference, whose driver returns
 * when the traversal is done).  wedge_cuda_run_async queues the whole
 * traversal -- the iteration loop runs on the device as with WEDGE_FLAG_GRAPH;
 * WEDGE_FLAG_TIMING is rejected -- and returns without waiting.
 * wedge_cuda_read_results_async queues the export of the last run's results
 * into page-locked host memory (cudaHostAlloc / cudaHostRegister; other memory
 * is rejected with WEDGE_ERR_ARG) on a second stream of the handle -- a kernel
 * writes them to a device staging buffer of 8 bytes per vertex (allocated on
 * the first call) and the copy engine moves them to the host -- so work
 * queued next on the handle's stream -- the next query, or other handles'
 * queries sharing that stream -- overlaps the transfer; a later run of the
 * same handle waits for the export before it overwrites the properties.
 * wedge_cuda_wait waits for both and returns the queued run's status and
 * statistics (stats may be NULL).  The host memory holds the results once
 * wedge_cuda_wait returns. */
int wedge_cuda_run_async(wedge_graph_t* g, int app, const wedge_params_t* params);
int wedge_cuda_read_results_async(wedge_graph_t* g, void* host_props, uint64_t bytes);
int wedge_cuda_wait(wedge_graph_t* g, wedge_stats_t* stats);
/* Waits only for the last wedge_cuda_read_results_async of the handle: its
 * host memory holds the results on return, while work queued after it (the
 * next queries on a shared stream) keeps running.  A pipelined host waits here
 * for query i's results after queueing query i+1.  Returns at once when no
 * export is pending. */
int wedge_cuda_wait_results(wedge_graph_t* g);

/* Queues the handle's work on a caller's stream (a cudaStream_t; NULL restores
 * the handle's own), after the work already queued on the previous one has
 * finished.  Handles sharing a stream run in the order their work was queued;
 * the traversal loops are still captured on the handle's own stream. */
int wedge_cuda_set_stream(wedge_graph_t* g, void* stream);

/* ---------------------------------------------------------------- knobs */

/* Launch parameters of the single-query engine, per handle (no counterpart in
 * the reference, whose kernels have none).  wedge_gb300/autotune.py times
 * them on a workload and stores the fastest per application; the Python layer
 * applies that table.  A knob set to WEDGE_KNOB_DEFAULT takes its environment
 * variable, else the built-in default.  Setting a knob releases the handle's
 * traversal state (the next run rebuilds it); results of the last run are
 * gone.  Out-of-range values return WEDGE_ERR_ARG. */
enum wedge_knob {
    WEDGE_KNOB_HUB_BYTES = 0,    /* shared-memory hub cache of the pulls, bytes: 0 (none) .. 196608, multiple
                                    of 16 (WEDGE_HUB_BYTES; default 65536); the device's limit applies */
    WEDGE_KNOB_PROBE_EDGES = 1,  /* BFS/CC per-destination probe window, in-edges: 1 .. 4096
                                    (WEDGE_PROBE_EDGES; default 16) */
    WEDGE_KNOB_SSSP_TILE = 2,    /* SSSP dense-pull tile, in-edges: 512 or 256 (WEDGE_SSSP_TILES512=1/0;
                                    default 512 from 2^23 in-edges, else 256); 512 needs byte-wide weights
                                    and in-edge positions, other graphs use 256 */
    WEDGE_KNOB_SSSP_NARROW = 3,  /* SSSP pulls gather a 32-bit copy of the distances (uint64 weights): 1, or
                                    0 (none), or a limit 2 .. 2^32-2 below which distances stay in 32 bits
                                    (the default limit is 2^32-1; lower ones test the switch to 64 bits)
                                    (WEDGE_SSSP_NARROW; default 1) */
    WEDGE_KNOBS = 4
};
#define WEDGE_KNOB_DEFAULT UINT64_MAX

int wedge_cuda_set_knob(wedge_graph_t* g, int knob, uint64_t value);
/* the value the next state build uses (after the environment and defaults) */
int wedge_cuda_get_knob(wedge_graph_t* g, int knob, uint64_t* value);

/* ---------------------------------------------------------------- shards */

/* Destination-range shards: the reference's NUMA split (graphdata.c:1050-1065:
 * edge vectors divided evenly; graphdata.c:656-689: each part's vertex range
 * ends at its last destination, rounded up to a 512-vertex boundary), one
 * shard per GPU.  A shard holds the in-edges of its destination range only
 * (grouped by ascending dst, as wedge_cuda_load_edges), over all vertices as
 * sources; global_outdeg[num_vertices] are the whole graph's out-degrees and
 * global_edges its edge count, so every shard numbers vertices alike and
 * takes the dense/Wedge decision on the whole graph's terms.  BFS, CC and
 * SSSP run phase by phase (wedge_cuda_run_phase): after each pull the host
 * combines the shards' properties (element-wise minimum) and pulled frontier
 * bitmaps (bitwise or; the shards' destinations are disjoint), imports them
 * into every shard, and hands every shard the summed changed mass. */
enum wedge_shard_state {
    WEDGE_SHARD_PROPS = 0,    /* one word per vertex in the engine's numbering: uint32 (BFS parent, CC label)
                                 or uint64 (SSSP distance) */
    WEDGE_SHARD_FRONTIER = 1  /* the bitmap of vertices the last pull changed, (V + 31) / 32 uint32 words */
};
int wedge_cuda_load_shard(uint64_t num_vertices, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                          const uint64_t* weights, int weight_kind, const uint64_t* global_outdeg,
                          uint64_t global_edges, wedge_graph_t** out);
/* copies a shard's state (enum wedge_shard_state) to host memory (import 0) or back from it (import 1) */
int wedge_cuda_shard_state(wedge_graph_t* g, int which, void* host, uint64_t bytes, int import);
/* after a pull and the import: the iteration's decision from the changed mass of all shards */
int wedge_cuda_shard_decide(wedge_graph_t* g, uint64_t global_mass, uint64_t threshold_pct);

/* ---------------------------------------------------------------- results */

/* per-iteration records of the last run (at most 4096 kept); *count receives the number
 * of iterations recorded, min(count, max_records) records are written */
int wedge_cuda_iteration_log(wedge_graph_t* g, wedge_iteration_record_t* out, uint64_t max_records,
                             uint64_t* count);

/* graph_vertex_props, one 64-bit word per vertex (see the header comment); bytes >= 8*V */
int wedge_cuda_read_results(wedge_graph_t* g, void* host_props, uint64_t bytes);
/* graph_vertex_outdegrees as uint64 counts; bytes >= 8*V */
int wedge_cuda_read_outdegrees(wedge_graph_t* g, uint64_t* host_outdeg, uint64_t bytes);
/* The -o output of the last run (source/main.c:112-150: one "%llu %s\n" line per vertex in
 * the format of execution_get_vertex_prop_string_*), written to `path`.  BFS, CC and
 * uint64 SSSP lines are formatted on the GPU (a length pass, a scan, a write pass) and
 * written with one fwrite; PageRank's %.4le and FP64 SSSP distances are formatted on the
 * host.  *gpu_formatted tells which; format_ms is the formatting time (both optional). */
int wedge_cuda_write_output(wedge_graph_t* g, const char* path, int* gpu_formatted, double* format_ms);

/* ---------------------------------------------------------------- learned scheduler */

/* No counterpart in the reference.  Loads a scheduler network (count =
 * WEDGE_SCHED_BLOB floats in host memory, layout above) that the
 * WEDGE_SCHED_LEARNED runs of g evaluate on the device after every pull: the
 * features of the next iteration go through the network, and the strategy with
 * the least predicted cost runs unless a feature lies outside [lo, hi] or the
 * predicted gain over the plain rule's choice is below the margin.  CC's first
 * pull stays dense (execution_cc.c:103), and so does every iteration 0. */
int wedge_cuda_set_scheduler(wedge_graph_t* g, const float* blob, uint64_t count);

/* Training and checking of a scheduler network with the engine's own CUDA
 * kernels on the current device.  X[n][16] features, Y[n][3] target log2 costs,
 * M[n][3] = 1 where the target was measured, else 0; the loss is the sum over
 * measured entries of (y - target)^2 divided by n.  Blobs are host memory of
 * WEDGE_SCHED_BLOB floats; mu/sd standardise the features inside the network. */
int wedge_mlp_forward(const float* blob, const float* X, uint64_t n, float* out /* [n][3] */);
int wedge_mlp_loss_grad(const float* blob, const float* X, const float* Y, const float* M, uint64_t n,
                        double* loss, float* grad /* [WEDGE_SCHED_PARAMS], d loss / d params */);
/* Adam on minibatches of `batch` samples in an order drawn from `seed`; blob
 * holds the initial parameters on entry and the trained ones on return. */
int wedge_mlp_train(float* blob, const float* X, const float* Y, const float* M, uint64_t n, uint32_t epochs,
                    uint32_t batch, float lr, uint64_t seed, double* final_loss);

/* ---------------------------------------------------------------- batched queries */

/* No counterpart in the reference, which runs one query per process.  Many
 * BFS and SSSP queries over many graphs run together in one persistent
 * cooperative kernel: every iteration of every unfinished query is split into
 * 32-edge chunks on one device work queue, and the Wedge frontiers of all
 * queries are built in the same pass, so small and large queries share the
 * GPU.  Results equal those of wedge_cuda_run on each query alone. */
typedef struct wedge_query {
    uint32_t graph;           /* index into the batch's graph array */
    int32_t app;              /* WEDGE_APP_BFS or WEDGE_APP_SSSP (SSSP needs a weighted graph) */
    uint64_t root;            /* the caller's vertex id; out of range selects 0 (main.c:81-85) */
} wedge_query_t;

typedef struct wedge_batch_tuning {
    uint32_t threshold_pct;   /* dense pull iff active out-edge mass > t% of the query's edges (0: 20) */
    uint32_t grab;            /* 32-edge chunks a warp takes from the queue at a time (0: 8) */
    uint32_t blocks_per_sm;   /* persistent blocks per SM, at most the occupancy limit (0: that limit) */
    uint32_t split;           /* out-degree above which the Wedge build expands a vertex with the whole
                                 warp instead of one lane (0: 32) */
} wedge_batch_tuning_t;

typedef struct wedge_batch_stats {
    double running_ms;        /* the persistent launch (and its setup kernels), CUDA events */
    uint64_t rounds;          /* iterations of the slowest query */
    uint64_t chunks_pulled;   /* queue items over all rounds */
    uint64_t iterations;      /* iterations summed over queries */
    uint32_t captured;        /* 1 if the run replayed a captured CUDA graph */
    uint32_t blocks;          /* persistent blocks */
} wedge_batch_stats_t;

typedef struct wedge_batch wedge_batch_t;

/* graphs: loaded handles on one device (kept alive by the caller until the batch is freed) */
int wedge_cuda_batch_create(wedge_graph_t* const* graphs, uint32_t num_graphs, const wedge_query_t* queries,
                            uint32_t num_queries, wedge_batch_t** out);
/* tuning may be NULL (defaults); flags: WEDGE_FLAG_GRAPH captures setup + launch once and replays it */
int wedge_cuda_batch_run(wedge_batch_t* b, const wedge_batch_tuning_t* tuning, uint32_t flags,
                         wedge_batch_stats_t* stats);
/* one query's graph_vertex_props (8 bytes per vertex of its graph, as wedge_cuda_read_results) */
int wedge_cuda_batch_read_result(wedge_batch_t* b, uint32_t query, void* host_props, uint64_t bytes);
/* iterations each query ran, host array of num_queries */
int wedge_cuda_batch_iterations(wedge_batch_t* b, uint32_t* host_iterations, uint32_t num_queries);
void wedge_cuda_batch_free(wedge_batch_t* b);

/* ---------------------------------------------------------------- allocation-free iteration */

/* No counterpart in the reference.  One PageRank iteration -- the edge pull
 * (perform_edge_pull_phase_pr) and the vertex phase -- for callers that cannot
 * allocate device memory, such as a host framework that owns every device
 * allocation through its own pool, or code that must not trigger a cudaMalloc in
 * the middle of its own stream work.  Nothing is allocated: the scratch lives in
 * a fixed static device array of about 6.3 MB that every GPU loading this
 * library holds until exit.  The caller owns all inputs and outputs, in device
 * memory:
 *   dst_off[num_dsts+1]  first in-edge of each destination that has in-edges
 *                        (strictly increasing, dst_off[num_dsts] == num_edges)
 *   dst_id[num_dsts]     vertex id of each such destination, ascending
 *   src[]                in-edge sources, 16-byte aligned, padded with
 *                        0xFFFFFFFF to a multiple of 128 entries
 *   outdeg[num_vertices] out-degree of every vertex
 *   rank_in, rank_out    [num_vertices] rank / outdegree' (graph_vertex_props of
 *                        PageRank); rank_out must not alias rank_in
 * damping <= 0 selects 0.875.  num_edges above WEDGE_NOALLOC_MAX_EDGES is
 * rejected with WEDGE_ERR_ARG.  Work is queued on `stream` (a cudaStream_t, NULL
 * for the default stream) and the call returns without waiting.  The first call
 * on a device looks up the scratch array's device address (make that first call
 * before any stream capture).  All calls share the one array: calls that
 * overlap on the GPU race and must be ordered by the caller.  The address is
 * kept for the life of the process: calls from a context other than the
 * device's primary context, or after a cudaDeviceReset, are not supported. */
#define WEDGE_NOALLOC_MAX_EDGES (1ull << 24)
int wedge_cuda_pr_iteration_noalloc(uint64_t num_vertices, uint64_t num_dsts, uint64_t num_edges,
                                    const uint64_t* dst_off, const uint32_t* dst_id, const uint32_t* src,
                                    const uint32_t* outdeg, const double* rank_in, double* rank_out,
                                    double damping, void* stream);

uint64_t wedge_cuda_num_vertices(const wedge_graph_t* g);
uint64_t wedge_cuda_num_edges(const wedge_graph_t* g);
/* the CUDA stream (cudaStream_t) the graph's kernels run on, as an opaque pointer */
void* wedge_cuda_stream(const wedge_graph_t* g);
/* graph_data_* teardown (the reference never frees); safe on NULL */
void wedge_cuda_free(wedge_graph_t* g);
const char* wedge_cuda_status_string(int status);
int wedge_cuda_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif
