// Shared definitions of the sm_103a edge-pull engine.
//
// Device layout of a loaded graph (all resident in HBM):
//   src[Epad]      uint32 in-edge sources, grouped by destination in file order,
//                  padded to a multiple of TILE with NONE32
//   w[Epad]        64-bit weight words (SSSP only; uint64 or IEEE double)
//   dst_id[Vne]    vertex id of compressed destination k (only vertices with
//                  in-degree > 0 are listed, ascending)
//   dst_off[Vne+1] first edge of compressed destination k
//   dst_start[Epad/32] one bit per in-edge: the first in-edge of its destination
//   tile_dst0[T+1] compressed destination owning edge 128*t (Vne where that
//                  edge is padding); pull tiles of 32*EPL edges index it with a stride
//   outdeg[V]      out-degree (graphdata.c:430-490)
//   csri_off[V+1], csri[E]  for every source, the in-edge position of each of
//                  its out-edges (its Wedge chunk of 32 in-edges = position / 32;
//                  chunk ids where Epad >= 2^32): the CSRI of graphdata.c:493-585
// A tile (128 consecutive in-edges) is the unit of work of one warp; a chunk
// (32 in-edges, one 128-byte line of sources) is the unit the Wedge frontier
// marks, i.e. the GPU form of the reference's frontier element of 4 edge
// vectors (include/configuration.h:19-24).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "wedge_cuda.h"

namespace wedge {

constexpr uint32_t TILE = 128;          // granularity of the tile index (tile_dst0)
constexpr uint32_t MAX_TILE_E = 512;    // largest pull tile; E is padded to a multiple of it
constexpr uint32_t CHUNK = 32;
constexpr uint32_t CHUNKS_PER_TILE = TILE / CHUNK;        // 4
constexpr uint32_t TILES_PER_WORD = 32 / CHUNKS_PER_TILE;  // 8 tiles per 32-bit chunk-bitmap word
constexpr uint32_t REGION_WORDS = 32;                      // chunk-bitmap words per summary bit
constexpr uint32_t TILES_PER_REGION = REGION_WORDS * TILES_PER_WORD;  // 256 tiles = 32768 in-edges
constexpr uint32_t PIECE = 256;                            // CSRI entries per Wedge-build work item
constexpr uint32_t BIG_LIST = 8;                           // longer CSRI lists go to warp-wide work items
constexpr uint32_t NONE32 = 0xFFFFFFFFu;
constexpr unsigned long long NONE64 = ~0ull;
constexpr uint32_t FULL = 0xFFFFFFFFu;

// pull strategies: every tile; the tiles of the Wedge frontier; every tile with
// gathers only from sources the previous pull changed (CC/SSSP; BFS = dense,
// whose gathers are frontier bits already)
enum : uint32_t { MODE_DENSE = 0, MODE_WEDGE = 1, MODE_FILTERED = 2 };

// per-block counters written by the pulls (NCNT slots per block)
// CNT_OCC: writes of 32-vertex words of the pull's output bitmap, counted once
// per distinct word of a warp's group (a word written by several warps counts
// once per warp): how clustered the changed vertices are, the GPU form of the
// reference's test of empty frontier groups (phase_edge_pull_bfs.c:244-246)
constexpr uint32_t NCNT = 9;
enum : uint32_t { CNT_MASS = 0, CNT_EDGES = 1, CNT_TILES = 2, CNT_DSTS = 3, CNT_ACT = 4, CNT_DEG0 = 5, CNT_DEG1 = 6,
                  CNT_DEG2 = 7, CNT_OCC = 8 };
// out-degree buckets of activated vertices (scheduler features): <= 4, <= 32, <= 256, more
__host__ __device__ constexpr uint32_t degree_bucket(uint32_t d) { return d <= 4u ? 0u : d <= 32u ? 1u : d <= 256u ? 2u : 3u; }
constexpr uint32_t LOG_CAP = 4096;  // iterations kept in the per-iteration log

// one iteration of the per-iteration log (the ITERATION_STATS record of
// execution_bfs.c:227-232, plus device counters)
struct IterRec {
    unsigned long long mass_in;    // active edges that chose this iteration's pull
    unsigned long long mass_out;   // changed-edge mass the pull produced
    unsigned long long edges;      // in-edges read
    unsigned long long tiles;      // tiles visited
    unsigned long long dsts;       // destinations in visited tiles
    unsigned long long activated;  // vertices activated
    unsigned int mode;             // MODE_DENSE / MODE_WEDGE / MODE_FILTERED
    unsigned int iter;
    float feat[16];                // scheduler features this iteration's mode was chosen on
    unsigned int learned;          // 1 if the scheduler network chose the mode
    unsigned int pad;
};

// Device control block of one traversal; read and written only by the
// engine's kernels (the host reads it back for statistics).
struct Ctrl {
    unsigned long long mass;           // changed out-edge mass of the last pull (phases.c:26-35)
    unsigned long long last_mass;      // mass that chose the current mode
    unsigned long long edges_scanned;  // in-edges read by pulls
    unsigned long long tiles_scanned;  // tiles visited by pulls
    unsigned long long threshold;      // |E| * t% / 100 (execution_bfs.c:132)
    unsigned long long dsts_scanned;   // destinations in visited tiles
    unsigned long long activated;      // vertices activated by pulls
    unsigned int items;                // Wedge-build work items appended by the last pull
    unsigned int need_n;               // tiles the probe listed for the dense tile pull (tile_list)
    unsigned int cand_n;               // BFS: candidate destinations the last Wedge build listed
    unsigned int tiles;                // length of the Wedge tile list
    unsigned int mode;                 // MODE_DENSE / MODE_WEDGE for the next pull
    unsigned int iter;                 // completed pulls
    unsigned int wedge_iters;          // pulls that used the Wedge frontier
    unsigned int done;                 // traversal finished
    unsigned int not_converged;        // iteration cap reached
    unsigned int max_iter;
    unsigned int sched;                // enum wedge_sched
    unsigned int parity;               // BFS frontier double-buffer parity
    unsigned int loop;                 // 1 while the traversal continues (CUDA-graph loop condition)
    unsigned int error;                // kernel-detected error (bounds)
    unsigned int pull_launches;
    unsigned int probe_iter;           // WEDGE_SCHED_PROBE: iteration whose mode is forced
    unsigned int probe_mode;
    unsigned int learned_iters;        // iterations whose mode the scheduler network chose
    unsigned int alist_n;              // vertices in the Wedge-build vertex list
    unsigned int pr_ticket;            // blocks of pr_total_kernel done (the last one resets it)
    unsigned int probe_edges;          // BFS/CC probe window of the next pull (in-edges per destination)
    unsigned int narrow_ovf;           // SSSP: a finite distance reached the 32-bit copy's limit; pulls gather the
                                       // 64-bit distances from then on
    unsigned int ovf_redo;             // SSSP: a pull dropped sums its 32-bit arithmetic could not hold: the next
                                       // pull is dense (64-bit) and the traversal does not stop before it
    double pr_total;                   // sum of all accumulators (phase_vertex_pr.c:161); compensated FP32:
                                       // the total the next iteration uses
    double pr_prev;                    // compensated FP32: the total the last iteration used
    double pr_sum;                     // PageRank Sum statistic
};

// Immutable graph, passed to kernels by value.
struct DevGraph {
    uint64_t V, E, Epad;
    uint64_t E_thr;            // edges the dense/Wedge threshold is a share of: E, or the whole graph's for a shard
    uint32_t Vne, T, nsplit, weight_kind;
    uint32_t dst_ident;        // dst_id[k] == k for every k (the vertices with in-edges are [0, Vne))
    uint32_t nwide;            // destinations spanning more than SPLIT_SERIAL tile boundaries (back of the split lists)
    uint32_t sym;              // every edge's reverse is an edge too: CC propagates engine ids (see cc_best_kernel)
    uint32_t csri_pos;         // csri holds in-edge positions (Epad < 2^32), else chunk ids
    uint32_t shard;            // a destination-range shard (wedge_cuda_load_shard)
    const uint32_t* src;
    const unsigned long long* w;
    const uint8_t* w8;         // the same weights in one byte each, when every weight is a uint64 below 256
    const uint32_t* dst_id;
    const unsigned long long* dst_off;
    const uint32_t* tile_dst0;
    const uint32_t* dst_start; // [Epad/32] bit p: in-edge p is the first of its destination
    const uint32_t* outdeg;
    const unsigned long long* csri_off;
    const uint32_t* csri;
    const uint32_t* split_k;   // compressed destinations whose in-edges span tiles ([T]: nsplit short
                               // ones from the front, nwide long ones from the back)
    const uint32_t* split_t0;  // their first tile
    const uint32_t* split_t1;  // their last tile
    const uint32_t* new2old;   // degree relabelling: engine id -> caller's id
    const uint32_t* old2new;   // caller's id -> engine id
};

// Mutable per-traversal state, passed to kernels by value.
struct DevState {
    uint32_t* prop32;              // BFS parent / CC label
    unsigned long long* prop64;    // SSSP distance (uint64 or double bits)
    uint32_t* dist32;              // SSSP, uint64 weights: the distances below narrow_lim in 32 bits (NONE32:
                                   // unreached or not below the limit), the array the pulls gather while
                                   // Ctrl::narrow_ovf is 0; or null
    uint32_t narrow_lim;           // distances the 32-bit copy holds: below this (2^32-1, or a smaller test limit)
    uint32_t narrow_sums;          // the 512-edge SSSP pull may sum in 32 bits (not on shards: see ovf_redo)
    double* rank;                  // PageRank FP64: rank / outdegree'
    double* acc;                   // PageRank accumulators (graph_vertex_accumulators)
    double* inv_od;                // PageRank 1 / outdegree' (outdegree, or N for dangling vertices)
    double* head_part;             // [T] partial sum of a split destination ending in tile t
    double* tail_part;             // [T] partial sum of a split destination continuing past tile t
    // compensated-FP32 PageRank (WEDGE_PREC_FP32C): see pr32_pull_kernel
    float* rank32;                 // [2][rstride] rank / outdegree', double-buffered by iteration parity
    float* inv32;                  // [V] 1 / outdegree' in FP32, negative for a dangling vertex (-1/N)
    uint64_t rstride;              // floats between the two rank buffers (V rounded up to 32)
    uint32_t* zlist;               // vertices without in-edges and with out-edges (their rank is the same constant)
    uint32_t* ilist;               // vertices without in-edges or out-edges (written once, after the last iteration)
    uint32_t nz, ni;
    uint32_t* psplit_k;            // destinations spanning pull tiles (PR32_TILE in-edges): short ones from the
    uint32_t* psplit_t0;           // front (pnsplit), long ones from the back (pnwide; entry pT-1-j)
    uint32_t* psplit_t1;
    uint32_t pnsplit, pnwide, pT;
    float2* phead;                 // [pT] (sum, compensation) of a split destination ending in tile t
    float2* ptail;                 // [pT] (sum, compensation) of a split destination continuing past tile t
    unsigned long long* shead;     // SSSP 512-edge pull: [pT] minimum of a split destination ending in tile t
    unsigned long long* stail;     // [pT] minimum of a split destination continuing past tile t (the split lists
                                   // psplit_* are those of the 512-edge tiles)
    double* pmass;                 // per-block partial sums of the non-dangling ranks (the next total rank)
    float* ovf_sum;                // [Vne] sums of the destinations in ovf_list, by compressed destination
    uint32_t* ovf_list;            // complete destinations past the staged slots of their tile (tile order)
    uint32_t novf;
    double* block_part;            // [grid] per-block sums of tile sums
    uint32_t* front0;              // V-bit frontier bitmaps (active / snapshot)
    uint32_t* front1;
    uint32_t* vis_c;               // Vne-bit: destination finished (BFS visited; CC label 0, the least label)
    uint32_t* tile_open;           // T-bit: tile still has an unfinished destination (BFS, CC)
    uint32_t* tile_need;           // T-bit: BFS tiles with in-edges the probe left to the tile pull
    uint32_t* cand;                // Vne-bit: BFS candidate destinations of the next Wedge pull (listed once)
    uint32_t* cand_list;           // [Vne] those candidates
    uint32_t* chunk_bits;          // Wedge frontier: one bit per chunk
    uint32_t* summary;             // one bit per region of REGION_WORDS chunk words (any chunk marked)
    unsigned long long* tile_list; // (tile << 32 | chunk mask) of the next Wedge pull
    uint2* items;                  // (vertex, piece) Wedge-build work items
    uint32_t* alist;               // vertices the last pull activated (Wedge build)
    uint32_t* cc_best;             // CC on a symmetric graph: least caller id of the component a label represents
    const uint32_t* cc_map;        // results only: CC labels are looked up here (engine ids not yet converted)
    Ctrl* ctrl;
    IterRec* log;                  // [LOG_CAP] per-iteration records
    double damping;
    uint32_t precision;
    uint32_t app;
    uint64_t root;
    uint32_t hub_n;                // elements of the gathered array cached in shared memory by dense pulls
    uint32_t hub_bytes;            // their bytes: the pulls' dynamic shared memory (a multiple of 16)
    uint32_t hub_tile;             // CC/SSSP: first tile whose destinations all have ids >= hub_n
    uint32_t hub_k;                // CC/SSSP: compressed destinations with ids < hub_n
    const float* net;              // scheduler network blob (WEDGE_SCHED_LEARNED), or null
    uint32_t push;                 // SSSP over in-edge positions: Wedge pulls relax the activated sources' out-edges
    uint32_t probe_edges;          // default BFS/CC probe window
};

}  // namespace wedge

// host-side handle (opaque to C callers)
struct wedge_graph {
    wedge::DevGraph g;
    wedge::DevState s;
    cudaStream_t stream;               // the stream the handle's work is queued on (own_stream or a caller's)
    cudaStream_t own_stream;
    cudaStream_t xstream;              // result exports of wedge_cuda_read_results_async (created on first use)
    cudaEvent_t ev_run;                // recorded after a run, before an asynchronous export
    cudaEvent_t ev_x;                  // recorded after an asynchronous export: later runs wait for it
    int x_pending;                     // an asynchronous export is queued (until wedge_cuda_wait)
    unsigned long long* xbuf;          // device staging of asynchronous exports (8 bytes per vertex, on first use)
    int pend_app;                      // run queued by wedge_cuda_run_async, reported by wedge_cuda_wait (-1 none)
    uint64_t pend_launches;
    uint32_t pend_iters;
    int device;
    int num_sms;
    int weight_kind;
    int built_app;                     // app whose state arrays are sized (-1 none)
    int last_app;                      // app of the last run (for read_results)
    int last_precision;
    uint32_t pull_grid;                // persistent grid of the pull kernels (one 1024-thread block per SM)
    uint32_t build_grid;
    uint32_t dst_grid;                 // dst_kernel grid (two 1024-thread blocks per SM)
    uint32_t hub_bytes;                // the hub cache's bytes
    uint32_t pull_smem;                // dynamic shared memory of the tile pulls (hub cache + staged minima)
    float* net;                        // device copy of the scheduler network (wedge_cuda_set_scheduler)
    // allocations owned by the handle
    void* allocs[32];
    int nallocs;
    void* state_allocs[32];
    int nstate;
    unsigned long long* h_ctrl;        // pinned mirror of Ctrl (host reads)
    cudaEvent_t ev[8];
    double* iter_pull_ms;              // [LOG_CAP] per-iteration times of a WEDGE_FLAG_TIMING run
    double* iter_wedge_ms;
    int last_timing;
    cudaGraphExec_t graph_exec;        // captured traversal
    cudaGraphExec_t pr_exec;           // captured PageRank iterations
    uint64_t pr_key;                   // (iterations, precision) of pr_exec
    int graph_app;
    int graph_key;
    int cc_pending;                    // CC labels are engine ids (symmetric graph, not yet converted)
    uint64_t knob[WEDGE_KNOBS];        // wedge_cuda_set_knob values (WEDGE_KNOB_DEFAULT: environment, else default)
};

namespace wedge {
// implemented in engine.cu, used by loaders in graph.cu
int build_from_device_edges(wedge_graph* h, uint64_t V, uint64_t E, uint32_t* d_src, uint32_t* d_dst,
                            unsigned long long* d_w, int weight_kind, const uint32_t* d_global_outdeg = nullptr);
int new_handle(wedge_graph** out);
void free_handle(wedge_graph* h);
int track(wedge_graph* h, void* p);
int cuda_status(cudaError_t e);
}  // namespace wedge

#define WEDGE_CHECK(call)                                          \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return wedge::cuda_status(e_);      \
    } while (0)
